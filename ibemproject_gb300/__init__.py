"""GB300-native (sm_103a) implementation of the 3D elastic spherical iBEM path.

The compute lives in ``libibem_gb300.so`` (CUDA kernels + C ABI, ``include/ibem_gb300.h``)
and its C++ host layer (``host/ibem_plugins.*``), which mirrors the reference's
integrator / BEMBuilder / systemSolver / postProcessor plugins.  This module loads the
library with ctypes and exposes the C ABI to Python callers (tests, the bench); device
buffers are passed as raw pointers (for example ``torch.Tensor.data_ptr()``).

There is no CPU path: every entry point raises if the library is not built or a call
fails.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libibem_gb300.so")

IBEM_OK, IBEM_ERR_ARG, IBEM_ERR_CUDA, IBEM_ERR_NOCONV, IBEM_ERR_TIMEOUT, IBEM_ERR_SINGULAR, IBEM_ERR_IO = range(7)
SOLVE_FP64, SOLVE_MIXED_IR, SOLVE_GMRES_BJ = 0, 1, 2

_c_dp = ctypes.POINTER(ctypes.c_double)
_c_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p
_i64 = ctypes.c_int64
_int = ctypes.c_int
_dbl = ctypes.c_double


class Material(ctypes.Structure):
    _fields_ = [("E0", ctypes.c_double), ("nu0", ctypes.c_double),
                ("E1", ctypes.c_double), ("nu1", ctypes.c_double)]


class SolveReport(ctypes.Structure):
    _fields_ = [("backward_error", ctypes.c_double), ("iterations", ctypes.c_int),
                ("info", ctypes.c_int), ("t_factor_ms", ctypes.c_double),
                ("t_solve_ms", ctypes.c_double)]


class Batch(ctypes.Structure):
    _fields_ = [("nseg", ctypes.c_int), ("seg_begin", ctypes.POINTER(ctypes.c_int)),
                ("centers_dev", ctypes.c_void_p), ("radius_dev", ctypes.c_void_p),
                ("mats", ctypes.POINTER(Material)), ("axes_dev", ctypes.c_void_p), ("quats_dev", ctypes.c_void_p)]


class MfOptions(ctypes.Structure):
    _fields_ = [("restart", ctypes.c_int), ("max_cycles", ctypes.c_int), ("max_outer", ctypes.c_int),
                ("tol", ctypes.c_double), ("inner_tol", ctypes.c_double), ("stepwise", ctypes.c_int)]


class MfReport(ctypes.Structure):
    _fields_ = [("rel_residual", ctypes.c_double), ("outer", ctypes.c_int), ("inner", ctypes.c_int),
                ("t_setup_ms", ctypes.c_double), ("t_solve_ms", ctypes.c_double)]


PRECOND_BLOCK_JACOBI, PRECOND_LEARNED, PRECOND_NEUMANN = 0, 1, 2
GEN_RSA, GEN_MC = 0, 1


class GenParams(ctypes.Structure):
    _fields_ = [("num", ctypes.c_int), ("r0", ctypes.c_double), ("rlo", ctypes.c_double), ("rhi", ctypes.c_double),
                ("vf", ctypes.c_double), ("gap", ctypes.c_double), ("method", ctypes.c_int),
                ("seed", ctypes.c_uint64), ("max_tries", ctypes.c_int64), ("sweeps", ctypes.c_int)]


class EllGenParams(ctypes.Structure):
    _fields_ = [("num", ctypes.c_int), ("a1", ctypes.c_double), ("a2lo", ctypes.c_double), ("a2hi", ctypes.c_double),
                ("a3lo", ctypes.c_double), ("a3hi", ctypes.c_double), ("vf", ctypes.c_double),
                ("gap", ctypes.c_double), ("seed", ctypes.c_uint64), ("max_tries", ctypes.c_int64),
                ("method", ctypes.c_int), ("sweeps", ctypes.c_int)]


class IbemError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"ibem status {status}: {msg}")
        self.status = status


# Every symbol the header declares, with its ctypes signature.
SIGNATURES = {
    "ibem_last_error": (ctypes.c_char_p, []),
    "ibem_layout_size": (_int, [_int]),
    "ibem_kernel_launches": (ctypes.c_longlong, []),
    "ibem_prof_enable": (None, [_int]),
    "ibem_prof_report": (_int, [ctypes.c_char_p, _int]),
    "ibem_e3d_pair_blocks": (_int, [_vp, _vp, _int, ctypes.POINTER(Material), _int, _vp, _i64, _i64, _i64, _vp]),
    "ibem_e3d_node_blocks": (_int, [_vp, _int, _vp, _vp, _int, ctypes.POINTER(Material), _int, _vp, _i64, _i64,
                                    _i64, _vp]),
    "ibem_e3d_bem_hg": (_int, [_vp, _int, _vp, _int, ctypes.POINTER(Material), _vp, _i64, _i64, _i64, _vp, _i64,
                               _i64, _i64, _vp]),
    "ibem_e3d_bem_to_incl": (_int, [_vp, _int, _vp, _int, _vp, _int, ctypes.POINTER(Material), _int, _vp, _i64,
                                    _i64, _vp, _i64, _i64, _i64, _vp]),
    "ibem_e3d_bc_plan": (_int, [_int, _int, _c_ip, _c_dp, _c_dp, _c_ip, _c_ip]),
    "ibem_e3d_apply_bc": (_int, [_int, _int, _i64, _vp, _vp, _vp, _vp, _vp, _i64, _vp, _i64, _vp, _i64, _vp, _vp]),
    "ibem_e3d_get_ut": (_int, [_int, _int, _i64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ibem_e3d_farfield_rhs": (_int, [_int, ctypes.POINTER(Material), _int, _c_dp, _vp, _vp]),
    "ibem_e3d_solve": (_int, [_int, _i64, _vp, _i64, _vp, _vp, _dbl, ctypes.POINTER(SolveReport), _vp]),
    "ibem_e3d_solve_bj": (_int, [_i64, _int, _vp, _i64, _vp, _vp, _dbl, ctypes.POINTER(SolveReport), _vp]),
    "ibem_gemm_sub_f32": (_int, [_i64, _i64, _i64, _vp, _i64, _vp, _i64, _vp, _i64, _vp]),
    "ibem_e3d_solve_noalloc": (_int, [_i64, _vp, _i64, _vp, _vp, ctypes.POINTER(SolveReport), _vp]),
    "ibem_selftest_bounded_wait": (_int, [_int, ctypes.c_longlong, _vp]),
    "ibem_e3d_field": (_int, [_vp, _int, _vp, _vp, _int, ctypes.POINTER(Material), _int, _vp, _vp, _int, _vp,
                              _int, _vp, _vp, _c_dp, _vp, _vp]),
    "ibem_e3d_field_form": (_int, [_int, _vp, _int, _vp, _vp, _int, ctypes.POINTER(Material), _int, _vp, _vp, _int,
                                   _vp, _int, _vp, _vp, _c_dp, _vp, _vp]),
    "ibem_e3d_field_grid": (_int, [_int, _c_dp, _c_dp, _c_ip, _vp, _vp, _int, ctypes.POINTER(Material), _int, _vp, _vp,
                                   _int, _vp, _int, _vp, _vp, _c_dp, _vp, _vp]),
    "ibem_e3d_run_host": (_int, [_int, _int, ctypes.POINTER(Material), _int, _c_dp, _int, _c_ip, _c_dp, _c_dp,
                                 _int, _c_dp, _c_dp, _int, _c_dp, _c_dp, _dbl, _c_dp, _c_dp,
                                 ctypes.POINTER(SolveReport)]),
    "ibem_e3d_run_dir": (_int, [ctypes.c_char_p, _int, _int, _dbl, ctypes.POINTER(SolveReport)]),
    "ibem_e3d_ell_pair_blocks": (_int, [_vp, _vp, _vp, _int, ctypes.POINTER(Material), _vp, _i64, _i64, _i64, _vp]),
    "ibem_e3d_ell_field": (_int, [_int, _vp, _int, _vp, _vp, _vp, _int, ctypes.POINTER(Material), _vp, _c_dp, _vp,
                                  _vp]),
    "ibem_e3d_run_host_ell": (_int, [_int, ctypes.POINTER(Material), _int, _c_dp, _c_dp, _c_dp, _int, _c_dp, _c_dp,
                                     _dbl, _c_dp, _c_dp, ctypes.POINTER(SolveReport)]),
    "ibem_e3d_mf_matvec": (_int, [ctypes.POINTER(Batch), _int, _vp, _vp, _vp]),
    "ibem_e3d_mf_solve": (_int, [ctypes.POINTER(Batch), _vp, _vp, _int, _vp, ctypes.POINTER(MfOptions),
                                 ctypes.POINTER(MfReport), _vp]),
    "ibem_e3d_batch_farfield_rhs": (_int, [ctypes.POINTER(Batch), _c_dp, _vp, _vp]),
    "ibem_e3d_mf_tuning": (_int, [ctypes.POINTER(Batch), _c_ip, _c_ip, _vp]),
    "ibem_e3d_mf_tile_shape": (_int, [ctypes.POINTER(Batch), _c_ip, _c_ip, _c_ip, _vp]),
    "ibem_e3d_mf_solve_layout": (_int, [ctypes.POINTER(Batch), _int, _vp, _vp, _int, _vp, ctypes.POINTER(MfOptions),
                                        ctypes.POINTER(MfReport), _vp]),
    "ibem_e3d_mf_matvec_layout": (_int, [ctypes.POINTER(Batch), _int, _int, _vp, _vp, _vp]),
    "ibem_e3d_effective_modulus": (_int, [ctypes.POINTER(Batch), _vp, _c_dp, _c_dp, _c_dp, _c_dp, _vp]),
    "ibem_e3d_batch_farfield_rhs_layout": (_int, [ctypes.POINTER(Batch), _int, _c_dp, _vp, _vp]),
    "ibem_e3d_batch_dense_solve": (_int, [ctypes.POINTER(Batch), _int, _int, _vp, _vp, _dbl,
                                          ctypes.POINTER(SolveReport), _vp]),
    "ibem_e3d_effective_modulus_layout": (_int, [ctypes.POINTER(Batch), _int, _vp, _c_dp, _c_dp, _c_dp, _c_dp,
                                                 _vp]),
    "ibem_e3d_run_host_mf": (_int, [ctypes.POINTER(Material), _int, _c_dp, _c_dp, _int, _c_dp, _c_dp, _int,
                                    ctypes.POINTER(ctypes.c_float), ctypes.POINTER(MfOptions), _c_dp, _c_dp,
                                    ctypes.POINTER(MfReport)]),
    "ibem_e3d_generate_spheres": (_int, [ctypes.POINTER(GenParams), _c_dp, _c_dp, _c_dp]),
    "ibem_e3d_generate_ellipsoids": (_int, [ctypes.POINTER(EllGenParams), _c_dp, _c_dp, _c_dp, _c_dp]),
    "ibem_e3d_sidecar_from_txt": (_int, [ctypes.c_char_p]),
    "ibem_e3d_sidecar_write": (_int, [ctypes.c_char_p, ctypes.POINTER(Material), _int, _c_dp, _int, _c_ip, _c_dp,
                                      _c_dp, _int, _c_dp, _c_dp, _int, _c_dp, _c_dp]),
    "ibem_e3d_case_sizes": (_int, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64)]),
    "ibem_e3d_read_case": (_int, [ctypes.c_char_p, ctypes.POINTER(Material), _c_dp, _c_ip, _c_dp, _c_dp, _c_dp,
                                  _c_dp, _c_dp, _c_dp]),
    "ibem_gnn_param_count": (_i64, []),
    "ibem_gnn_init_params": (_int, [_vp, ctypes.c_uint64, _vp]),
    "ibem_gnn_prepare": (_int, [ctypes.POINTER(Batch), _int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ibem_gnn_loss_grad": (_int, [_int, _vp, _vp, _vp, _int, _vp, _vp, _vp, _c_dp, _vp, _vp]),
    "ibem_gnn_edge_weights": (_int, [_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "ibem_gnn_adamw": (_int, [_i64, _vp, _vp, _vp, _vp, _int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                              ctypes.c_float, ctypes.c_float, _vp]),
    "ibem_gnn_train": (_int, [ctypes.POINTER(Batch), _int, _vp, _vp, _vp, _int, ctypes.c_float, ctypes.c_float,
                              _c_dp, _vp]),
}

_lib = None


def lib():
    """Load libibem_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with ibemproject_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != IBEM_OK:
        raise IbemError(status, lib().ibem_last_error().decode(errors="replace"))


def material(E0, nu0, E1, nu1) -> Material:
    return Material(E0, nu0, E1, nu1)


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_c_dp)


def _ip(a: np.ndarray):
    return a.ctypes.data_as(_c_ip)


def run_host(case, layout: int = 78, form: int = SOLVE_FP64, tol: float = 1e-12):
    """Whole pipeline through the host-buffer C ABI: returns (X, stress, report)."""
    m = material(case.E0, case.nu0, case.E1, case.nu1)
    N = 3 * case.NN + layout * case.num
    X = np.zeros(N)
    S = np.zeros((case.nump, 6))
    rep = SolveReport()
    f64 = lambda a, shape: np.ascontiguousarray(a if a is not None and np.size(a) else np.zeros(shape),
                                                dtype=np.float64)
    nodes = f64(case.nodes, 3)
    conn = np.ascontiguousarray(case.conn if case.NE else np.zeros(4, np.int32), dtype=np.int32)
    bc = f64(case.bc, 2)
    tbc = f64(case.tbc, 24)
    cen = f64(case.centers, 3)
    rad = f64(case.radius, 1)
    pts = f64(case.points, 3)
    sig = np.ascontiguousarray(case.sig_inf, dtype=np.float64) if case.sig_inf is not None else None
    check(lib().ibem_e3d_run_host(layout, form, ctypes.byref(m), case.NN, _dp(nodes), case.NE, _ip(conn),
                                  _dp(bc), _dp(tbc), case.num, _dp(cen), _dp(rad), case.nump, _dp(pts),
                                  _dp(sig) if sig is not None else None, tol, _dp(X), _dp(S),
                                  ctypes.byref(rep)))
    return X, S, rep


def run_host_mf(case, precond: int = PRECOND_LEARNED, params=None, tol: float = 1e-10):
    """Boundary-free far-field pipeline, matrix-free solve, through the host-buffer C ABI:
    returns (X, stress, MfReport).  params: host float32 array (learned form)."""
    m = material(case.E0, case.nu0, case.E1, case.nu1)
    N = 24 * case.num
    X = np.zeros(N)
    S = np.zeros((case.nump, 6))
    rep = MfReport()
    cen = np.ascontiguousarray(case.centers, dtype=np.float64)
    rad = np.ascontiguousarray(case.radius, dtype=np.float64)
    pts = np.ascontiguousarray(case.points if case.nump else np.zeros((1, 3)), dtype=np.float64)
    sig = np.ascontiguousarray(case.sig_inf, dtype=np.float64)
    prm, hold = None, None
    if params is not None:
        hold = np.ascontiguousarray(params, dtype=np.float32)   # kept alive across the call
        prm = hold.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    opt = MfOptions(0, 0, 0, tol, 0.0)
    check(lib().ibem_e3d_run_host_mf(ctypes.byref(m), case.num, _dp(cen), _dp(rad), case.nump, _dp(pts), _dp(sig),
                                     precond, prm, ctypes.byref(opt), _dp(X), _dp(S), ctypes.byref(rep)))
    return X, S, rep


def run_host_ell(case, form: int = SOLVE_FP64, tol: float = 1e-12):
    """Boundary-free ellipsoid pipeline (case.axes, case.quats set) through the host-buffer
    C ABI: returns (X, stress, report)."""
    m = material(case.E0, case.nu0, case.E1, case.nu1)
    N = 24 * case.num
    X = np.zeros(N)
    S = np.zeros((max(case.nump, 1), 6))
    rep = SolveReport()
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    cen, ax, qt = f64(case.centers), f64(case.axes), f64(case.quats)
    pts = f64(case.points if case.nump else np.zeros((1, 3)))
    sig = f64(case.sig_inf)
    check(lib().ibem_e3d_run_host_ell(form, ctypes.byref(m), case.num, _dp(cen), _dp(ax), _dp(qt), case.nump, _dp(pts),
                                      _dp(sig), tol, _dp(X), _dp(S), ctypes.byref(rep)))
    return X, S[:case.nump], rep


def run_dir(path: str, layout: int = 78, form: int = SOLVE_FP64, tol: float = 1e-12) -> SolveReport:
    rep = SolveReport()
    check(lib().ibem_e3d_run_dir(path.encode(), layout, form, tol, ctypes.byref(rep)))
    return rep


def sidecar_from_txt(path: str) -> None:
    """Write path/case.ibemb from the directory's text files (ibem_e3d_sidecar_from_txt)."""
    check(lib().ibem_e3d_sidecar_from_txt(path.encode()))


def read_case_native(path: str):
    """The inputs of a case directory as the library reads them (the side-car when it is at
    least as new as the text files): returns (cases.Case, read_from_side_car)."""
    from . import cases
    sz = (ctypes.c_int64 * 6)()
    check(lib().ibem_e3d_case_sizes(path.encode(), sz))
    NN, NE, num, nump, has_ff, from_sc = (int(v) for v in sz)
    m = Material()
    nodes, bc = np.zeros((NN, 3)), np.zeros((3 * NN, 2))
    conn, tbc = np.zeros((NE, 4), np.int32), np.zeros((NE, 24))
    cen, rad, pts, sig = np.zeros((num, 3)), np.zeros(num), np.zeros((nump, 3)), np.zeros(6)
    check(lib().ibem_e3d_read_case(path.encode(), ctypes.byref(m), _dp(nodes), _ip(conn), _dp(bc), _dp(tbc),
                                   _dp(cen), _dp(rad), _dp(pts), _dp(sig)))
    c = cases.Case(m.E0, m.nu0, m.E1, m.nu1, nodes, conn, bc, tbc, cen, rad, pts, sig if has_ff else None)
    return c, bool(from_sc)


def bc_plan(case):
    ucol = np.zeros(3 * case.NN, dtype=np.int32)
    tcol = np.zeros(12 * case.NE, dtype=np.int32)
    conn = np.ascontiguousarray(case.conn, dtype=np.int32)
    check(lib().ibem_e3d_bc_plan(case.NN, case.NE, _ip(conn), _dp(np.ascontiguousarray(case.bc, dtype=np.float64)),
                                 _dp(np.ascontiguousarray(case.tbc, dtype=np.float64)), _ip(ucol), _ip(tcol)))
    return ucol, tcol


def prof_report() -> dict:
    """Phase timings recorded since the last ibem_prof_enable (see include/ibem_gb300.h)."""
    import json
    buf = ctypes.create_string_buffer(1 << 16)
    lib().ibem_prof_report(buf, len(buf))
    return json.loads(buf.value.decode())
