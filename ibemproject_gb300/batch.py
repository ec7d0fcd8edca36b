"""Python side of the matrix-free solver and the learned preconditioner
(``ibem_e3d_mf_*``, ``ibem_gnn_*`` in include/ibem_gb300.h).

A :class:`DeviceBatch` holds several boundary-free sphere microstructures on the device
(concatenated centres and radii, torch tensors used as plain device memory) and the
``ibem_e3d_batch`` record that the C ABI reads.  Every computation runs in
libibem_gb300.so; this module only moves arrays and fills records.

Scaled system (the one the preconditioner and the training pairs live in): with a_p the
radius of particle p and mu0 the matrix shear modulus of its realisation,
    As = Dr A Dc,  Dr = diag(a_p^o / mu0),  Dc = diag(a_p^-o),
o = 1 on the 18 first-order unknowns of a particle and 0 on its 6 zeroth-order ones.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import (Batch, IbemError, Material, MfOptions, MfReport, PRECOND_BLOCK_JACOBI, PRECOND_LEARNED,
               PRECOND_NEUMANN, SOLVE_FP64, SOLVE_MIXED_IR, SolveReport, check, lib)

NU = 24
KNN = 16
NODE_FEATS, EDGE_FEATS = 10, 7


def _ptr(t) -> int:
    return t.data_ptr()


def _linear(batch, layouts=(NU,)) -> None:
    if getattr(batch, "ellipsoids", False):
        raise ValueError("the matrix-free solver and the learned preconditioner take spheres; "
                         "solve ellipsoid batches with dense_batch_solve")
    if batch.layout not in layouts:
        raise ValueError(f"this matrix-free call takes layout {' or '.join(str(v) for v in layouts)}, "
                         f"not {batch.layout}")


class DeviceBatch:
    """Realisations (each a cases.Case of the far-field kind) resident on `device`, with
    `layout` unknowns per particle (24: the matrix-free solver's; 60 or 78: quadratic
    eigenstrain, solved by dense_batch_solve)."""

    def __init__(self, cases_list, device="cuda", layout: int = NU):
        import torch
        self.cases = list(cases_list)
        self.layout = int(layout)
        counts = [c.num for c in self.cases]
        self.seg_begin = np.zeros(len(counts) + 1, dtype=np.int32)
        self.seg_begin[1:] = np.cumsum(counts)
        self.num = int(self.seg_begin[-1])
        self.N = self.layout * self.num
        cen = np.concatenate([np.asarray(c.centers, dtype=np.float64).reshape(-1, 3) for c in self.cases])
        rad = np.concatenate([np.asarray(c.radius, dtype=np.float64) for c in self.cases])
        self.centers_host, self.radius_host = cen, rad
        self.centers = torch.from_numpy(cen.copy()).to(device)
        self.radius = torch.from_numpy(rad.copy()).to(device)
        self.mats = (Material * len(self.cases))(*[Material(c.E0, c.nu0, c.E1, c.nu1) for c in self.cases])
        # ellipsoids: every realisation carries semi-axes and quaternions (a batch is all
        # spheres or all ellipsoids)
        self.ellipsoids = all(getattr(c, "axes", None) is not None for c in self.cases) and bool(self.cases)
        self.axes = self.quats = None
        if self.ellipsoids:
            self.axes = torch.from_numpy(np.concatenate([np.asarray(c.axes, dtype=np.float64) for c in self.cases])).to(
                device)
            self.quats = torch.from_numpy(np.concatenate([np.asarray(c.quats, dtype=np.float64)
                                                          for c in self.cases])).to(device)
        self.rec = Batch(len(self.cases), self.seg_begin.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                         _ptr(self.centers), _ptr(self.radius), self.mats,
                         _ptr(self.axes) if self.ellipsoids else None, _ptr(self.quats) if self.ellipsoids else None)
        self.device = device

    @property
    def nseg(self) -> int:
        return len(self.cases)

    def ref(self):
        return ctypes.byref(self.rec)

    def seg_rows(self, s: int) -> slice:
        return slice(self.layout * int(self.seg_begin[s]), self.layout * int(self.seg_begin[s + 1]))

    def scalings(self):
        """(Dr, Dc) as host arrays of length N."""
        mu0 = np.repeat([c.E0 / (2 * (1 + c.nu0)) for c in self.cases], np.diff(self.seg_begin))
        o = np.zeros(self.layout)   # eigenstrain order of each unknown
        o[6:] = 1.0
        o[24:] = 2.0
        a = self.radius_host[:, None]
        dr = (a ** o) / mu0[:, None]
        dc = a ** (-o)
        return dr.ravel(), dc.ravel()

    def volumes(self):
        """Cell volume of each realisation: the cube that holds its sample grid, or the box
        of its centres grown by the largest radius when it has no grid."""
        out = []
        for c in self.cases:
            if c.nump:
                lo, hi = c.points.min(axis=0), c.points.max(axis=0)
                n = round(c.nump ** (1.0 / 3.0))
                h = (hi - lo) / max(n - 1, 1)
                side = (hi - lo) + h
            else:
                side = np.ptp(c.centers, axis=0) + 2 * c.radius.max()
            out.append(float(np.prod(side)))
        return np.array(out)


def farfield_rhs(batch: DeviceBatch, sig_inf):
    import torch
    b = torch.zeros(batch.N, dtype=torch.float64, device=batch.device)
    sig = np.ascontiguousarray(sig_inf, dtype=np.float64)
    check(lib().ibem_e3d_batch_farfield_rhs_layout(batch.ref(), batch.layout,
                                                   sig.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), _ptr(b),
                                                   None))
    return b


def dense_batch_solve(batch: DeviceBatch, b, form: int = SOLVE_MIXED_IR, tol: float = 1e-10, x=None):
    """Dense solves of every realisation (ibem_e3d_batch_dense_solve, the batch's layout):
    returns (x, list of SolveReport)."""
    import torch
    if x is None:
        x = torch.zeros_like(b)
    reps = (SolveReport * batch.nseg)()
    check(lib().ibem_e3d_batch_dense_solve(batch.ref(), batch.layout, form, _ptr(b), _ptr(x), tol, reps, None))
    return x, list(reps)


def matvec(batch: DeviceBatch, x, precision: int = 64):
    """y = A x without storing A (ibem_e3d_mf_matvec_layout, the batch's layout 24 or 60)."""
    _linear(batch, (NU, 60))
    import torch
    y = torch.empty_like(x)
    check(lib().ibem_e3d_mf_matvec_layout(batch.ref(), batch.layout, precision, _ptr(x), _ptr(y), None))
    torch.cuda.synchronize()
    return y


def solve(batch: DeviceBatch, b, precond: int = PRECOND_BLOCK_JACOBI, params=None, tol: float = 1e-10,
          inner_tol: float = 1e-5, restart: int = 50, max_outer: int = 8, max_cycles: int = 20, x=None,
          stepwise: bool = False):
    """Matrix-free solve of every realisation (the batch's layout: 24, or 60 with the
    block-Jacobi preconditioner): returns (x, list of MfReport).  stepwise: launch each Arnoldi
    step from the host instead of one captured CUDA graph per GMRES cycle."""
    _linear(batch, (NU, 60))
    import torch
    if x is None:
        x = torch.zeros_like(b)
    reps = (MfReport * batch.nseg)()
    opt = MfOptions(restart, max_cycles, max_outer, tol, inner_tol, int(stepwise))
    check(lib().ibem_e3d_mf_solve_layout(batch.ref(), batch.layout, _ptr(b), _ptr(x), precond,
                                         _ptr(params) if params is not None else None, ctypes.byref(opt), reps,
                                         None))
    return x, list(reps)


def tuning(batch: DeviceBatch):
    """(source slices of the FP32 product, of the double-float / FP64 products) chosen by the
    library's autotuner for this batch's shape."""
    _linear(batch)
    a, b = ctypes.c_int(0), ctypes.c_int(0)
    check(lib().ibem_e3d_mf_tuning(batch.ref(), ctypes.byref(a), ctypes.byref(b), None))
    return a.value, b.value


def tile_shape(batch: DeviceBatch):
    """(targets per CTA, persistent launch 0/1, source slices) of the FP32 product chosen by
    the library's autotuner for this batch's shape."""
    _linear(batch)
    t, p, h = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
    check(lib().ibem_e3d_mf_tile_shape(batch.ref(), ctypes.byref(t), ctypes.byref(p), ctypes.byref(h), None))
    return t.value, p.value, h.value


def effective_modulus(batch: DeviceBatch, x, sig_inf, volume=None):
    """(E_eff per realisation, mean strain nseg x 6)."""
    volume = np.ascontiguousarray(batch.volumes() if volume is None else volume, dtype=np.float64)
    sig = np.ascontiguousarray(sig_inf, dtype=np.float64)
    eps = np.zeros((batch.nseg, 6))
    e = np.zeros(batch.nseg)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    check(lib().ibem_e3d_effective_modulus_layout(batch.ref(), batch.layout, _ptr(x), dp(volume), dp(sig), dp(eps),
                                                  dp(e), None))
    return e, eps


def dense_system(case, device="cuda", layout: int = NU):
    """The matrix of one realisation, assembled by ibem_e3d_pair_blocks (FP64, column-major
    N x N, as a torch tensor whose transpose view is row-major)."""
    import torch
    n = layout * case.num
    A = torch.zeros((n, n), dtype=torch.float64, device=device)  # column-major: A[c, r]
    cen = torch.from_numpy(np.ascontiguousarray(case.centers, dtype=np.float64)).to(device)
    rad = torch.from_numpy(np.ascontiguousarray(case.radius, dtype=np.float64)).to(device)
    m = Material(case.E0, case.nu0, case.E1, case.nu1)
    check(lib().ibem_e3d_pair_blocks(_ptr(cen), _ptr(rad), case.num, ctypes.byref(m), layout, _ptr(A), n, 0, 0, None))
    torch.cuda.synchronize()
    return A  # storage is column-major: element (r, c) is A[c, r]


def dense_solve(case, b_seg, device="cuda", layout: int = NU):
    """Plain FP64 LU solve (ibem_e3d_solve, IBEM_SOLVE_FP64) of one realisation."""
    import torch
    A = dense_system(case, device, layout)
    n = A.shape[0]
    x = torch.zeros(n, dtype=torch.float64, device=device)
    rep = SolveReport()
    check(lib().ibem_e3d_solve(SOLVE_FP64, n, _ptr(A), n, _ptr(b_seg.contiguous()), _ptr(x), 1e-12,
                               ctypes.byref(rep), None))
    return x


def training_pairs(batch: DeviceBatch, nrhs: int, seed: int = 0):
    """Residual / correction pairs of the scaled system made by the plain FP64 solver:
    r_hat ~ N(0, 1) per entry, e_hat = As^-1 r_hat (solving A e = Dr^-1 r_hat with the
    FP64 LU, e_hat = Dc^-1 e).  Returns two (nrhs, N) FP64 device tensors."""
    _linear(batch)
    import torch
    rng = np.random.default_rng(seed)
    dr, dc = batch.scalings()
    R = rng.standard_normal((nrhs, batch.N))
    E = np.zeros_like(R)
    for s, c in enumerate(batch.cases):
        rows = batch.seg_rows(s)
        for q in range(nrhs):
            r = torch.from_numpy(R[q, rows] / dr[rows]).to(batch.device)
            e = dense_solve(c, r, batch.device).cpu().numpy()
            E[q, rows] = e / dc[rows]
    return (torch.from_numpy(R).to(batch.device), torch.from_numpy(E).to(batch.device))


def training_pairs_mf(batch: DeviceBatch, nrhs: int, seed: int = 0, tol: float = 1e-10):
    """The pairs of training_pairs for microstructures too large for the dense LU (a
    2,000-sphere system is 60 s in FP64): e_hat = As^-1 r_hat from the matrix-free solver
    with block-Jacobi preconditioning and FP64 refinement to relative residual tol, i.e.
    ||r_hat - As e_hat|| <= tol ||r_hat|| per realisation."""
    import torch
    _linear(batch)
    rng = np.random.default_rng(seed)
    dr, dc = batch.scalings()
    R = torch.from_numpy(rng.standard_normal((nrhs, batch.N))).to(batch.device)
    E = torch.empty_like(R)
    drt = torch.from_numpy(dr).to(batch.device)
    dct = torch.from_numpy(dc).to(batch.device)
    for q in range(nrhs):
        x, _ = solve(batch, (R[q] / drt).contiguous(), PRECOND_BLOCK_JACOBI, tol=tol)
        E[q] = x / dct
    return R, E


# ------------------------------------------------------------------ learned preconditioner
def param_count() -> int:
    return int(lib().ibem_gnn_param_count())


def init_params(seed: int = 0, device="cuda"):
    import torch
    p = torch.zeros(param_count(), dtype=torch.float32, device=device)
    check(lib().ibem_gnn_init_params(_ptr(p), seed, None))
    return p


def prepare(batch: DeviceBatch, r_hat=None, e_hat=None):
    """Graph, features and (with pairs) the training projections z, u; dict of tensors."""
    _linear(batch)
    import torch
    dev = batch.device
    E = batch.num * KNN
    nrhs = 0 if r_hat is None else int(r_hat.shape[0])
    out = {
        "nbr": torch.empty(E, dtype=torch.int32, device=dev),
        "xn": torch.empty(batch.num * NODE_FEATS, dtype=torch.float32, device=dev),
        "ef": torch.empty(E * EDGE_FEATS, dtype=torch.float32, device=dev),
        "z": torch.empty(max(nrhs, 1) * batch.N, dtype=torch.float32, device=dev),
        "u": torch.empty(max(nrhs, 1) * E * 2 * NU, dtype=torch.float32, device=dev),
        "nrhs": nrhs,
    }
    check(lib().ibem_gnn_prepare(batch.ref(), nrhs, _ptr(r_hat) if nrhs else None, _ptr(e_hat) if nrhs else None,
                                 _ptr(out["nbr"]), _ptr(out["xn"]), _ptr(out["ef"]), _ptr(out["z"]),
                                 _ptr(out["u"]), None))
    torch.cuda.synchronize()
    return out


def loss_grad(prep: dict, num: int, params):
    import torch
    g = torch.empty_like(params)
    loss = ctypes.c_double(0.0)
    check(lib().ibem_gnn_loss_grad(num, _ptr(prep["nbr"]), _ptr(prep["xn"]), _ptr(prep["ef"]), prep["nrhs"],
                                   _ptr(prep["z"]), _ptr(prep["u"]), _ptr(params), ctypes.byref(loss), _ptr(g),
                                   None))
    torch.cuda.synchronize()
    return loss.value, g


def edge_weights(prep: dict, num: int, params):
    """(w_e, alpha_e) of every edge, num*16 x 2 flattened."""
    import torch
    w = torch.empty(num * KNN * 2, dtype=torch.float32, device=params.device)
    check(lib().ibem_gnn_edge_weights(num, _ptr(prep["nbr"]), _ptr(prep["xn"]), _ptr(prep["ef"]), _ptr(params),
                                      _ptr(w), None))
    torch.cuda.synchronize()
    return w


def adamw(params, grad, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
    import torch
    check(lib().ibem_gnn_adamw(params.numel(), _ptr(params), _ptr(grad), _ptr(m), _ptr(v), step, lr, beta1, beta2,
                               eps, weight_decay, None))
    torch.cuda.synchronize()


def train(batch: DeviceBatch, r_hat, e_hat, params, steps: int, lr: float = 2e-3, weight_decay: float = 0.0):
    """Full-batch training on the GPU (ibem_gnn_train); returns the loss history."""
    _linear(batch)
    hist = np.zeros(steps + 1)
    check(lib().ibem_gnn_train(batch.ref(), int(r_hat.shape[0]), _ptr(r_hat), _ptr(e_hat), _ptr(params), steps, lr,
                               weight_decay, hist.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None))
    return hist


__all__ = ["DeviceBatch", "farfield_rhs", "dense_batch_solve", "matvec", "solve", "tuning", "effective_modulus",
           "dense_system", "dense_solve",
           "training_pairs", "training_pairs_mf", "param_count", "init_params", "prepare", "loss_grad", "edge_weights", "adamw", "train",
           "PRECOND_BLOCK_JACOBI", "PRECOND_LEARNED", "PRECOND_NEUMANN", "IbemError"]
