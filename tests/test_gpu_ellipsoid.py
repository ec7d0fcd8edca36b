"""Ellipsoidal inclusions on the GPU, through the C ABI, against the host build of the same
evaluator (tests/hostgen/hostell.cpp; pinned to the oracle's volume quadrature, Mura's
interior tensor and the reference's sphere and spheroid formulas in
tests/test_ellipsoid_host.py) and against the sphere entry points in the sphere limit.
Tolerances: matrix entries 1e-12 of the block maximum; eigenstrains and stresses 1e-9 (FP64
form) and 1e-8 (mixed form) of the largest entry."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, scaled_err

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

HG = os.path.join(ROOT, "tests", "hostgen")
SO = os.path.join(HG, "_build", "libhostell.so")
_dp = ctypes.POINTER(ctypes.c_double)


def d(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_dp)


@pytest.fixture(scope="module")
def g():
    import ibemproject_gb300 as g
    g.lib()
    return g


@pytest.fixture(scope="module")
def he():
    os.makedirs(os.path.dirname(SO), exist_ok=True)
    subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-I",
                    os.path.join(ROOT, "ibemproject_gb300", "csrc"), "-o", SO, os.path.join(HG, "hostell.cpp")],
                   check=True)
    return ctypes.CDLL(SO)


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def P(t):
    return ctypes.c_void_p(t.data_ptr())


def ell_matrix(g, c):
    N = 24 * c.num
    At = torch.zeros((N, N), dtype=torch.float64, device="cuda")
    m = g.material(c.E0, c.nu0, c.E1, c.nu1)
    cen, ax, qt = dev(c.centers), dev(c.axes), dev(c.quats)
    g.check(g.lib().ibem_e3d_ell_pair_blocks(P(cen), P(ax), P(qt), c.num, ctypes.byref(m), P(At), N, 0, 0, None))
    torch.cuda.synchronize()
    return At.cpu().numpy().T   # row-major view of the column-major matrix


def host_block(he, c, s, h):
    out = np.zeros(576)
    he.he_block24(d(c.centers[s] - c.centers[h]), d(c.quats[h]), d(c.axes[h]),
                  *[ctypes.c_double(v) for v in (c.E0, c.nu0, c.E1, c.nu1)], int(s == h), d(out))
    return out.reshape(24, 24)


def test_pair_blocks_match_host_evaluator(g, he):
    from ibemproject_gb300 import cases
    c = cases.ellipsoid_case(37, vf=0.1, seed=3)   # 37: a ragged last warp of targets
    A = ell_matrix(g, c)
    rng = np.random.default_rng(0)
    pairs = [(s, s) for s in range(3)] + [tuple(rng.integers(0, c.num, 2)) for _ in range(40)] + [(36, 0), (0, 36)]
    for s, h in pairs:
        want = host_block(he, c, s, h)
        got = A[24 * s:24 * s + 24, 24 * h:24 * h + 24]
        assert scaled_err(got, want) < 1e-12, (s, h)


def test_sphere_limit_matches_sphere_blocks(g):
    from ibemproject_gb300 import cases
    c = cases.farfield_case(num=30, r0=0.05, vf=0.12, grid=0, seed=9)
    c.axes = np.repeat(c.radius[:, None], 3, axis=1)
    q = np.random.default_rng(1).normal(size=(c.num, 4))
    c.quats = q / np.linalg.norm(q, axis=1, keepdims=True)
    A_ell = ell_matrix(g, c)
    N = 24 * c.num
    At = torch.zeros((N, N), dtype=torch.float64, device="cuda")
    m = g.material(c.E0, c.nu0, c.E1, c.nu1)
    cen, rad = dev(c.centers), dev(c.radius)
    g.check(g.lib().ibem_e3d_pair_blocks(P(cen), P(rad), c.num, ctypes.byref(m), 24, P(At), N, 0, 0, None))
    torch.cuda.synchronize()
    A_sph = At.cpu().numpy().T
    for s in range(c.num):
        for h in range(c.num):
            blk = A_sph[24 * s:24 * s + 24, 24 * h:24 * h + 24]
            assert scaled_err(A_ell[24 * s:24 * s + 24, 24 * h:24 * h + 24], blk) < 1e-12


@pytest.mark.parametrize("form,tol", [(0, 1e-9), (1, 1e-8)])
def test_pipeline_against_host_assembled_solve(g, he, form, tol):
    """run_host_ell (assembly, right-hand side, dense solve, stresses) against a numpy solve
    of the system assembled by the host evaluator, and stresses summed by it."""
    from ibemproject_gb300 import cases
    c = cases.ellipsoid_case(24, vf=0.1, seed=7, grid=3)
    X, S, rep = g.run_host_ell(c, form=form, tol=1e-14)
    N = 24 * c.num
    A = np.zeros((N, N))
    for s in range(c.num):
        for h in range(c.num):
            A[24 * s:24 * s + 24, 24 * h:24 * h + 24] = host_block(he, c, s, h)
    m = g.material(c.E0, c.nu0, c.E1, c.nu1)
    bt = torch.zeros(N, dtype=torch.float64, device="cuda")
    g.check(g.lib().ibem_e3d_farfield_rhs(c.num, ctypes.byref(m), 24, d(c.sig_inf), P(bt), None))
    torch.cuda.synchronize()
    Xh = np.linalg.solve(A, bt.cpu().numpy())
    assert scaled_err(X, Xh) < tol
    # stresses: remote stress + C0 : (sum of the strains of every ellipsoid - local eigenstrain)
    mu0 = c.E0 / (2 * (1 + c.nu0))
    lam0 = 2 * mu0 * c.nu0 / (1 - 2 * c.nu0)
    Sh = np.zeros((c.nump, 6))
    for i, p in enumerate(c.points):
        e = np.zeros(6)
        inside = -1
        for h in range(c.num):
            if he.he_strain24(d(p - c.centers[h]), d(c.quats[h]), d(c.axes[h]),
                              *[ctypes.c_double(v) for v in (c.E0, c.nu0, c.E1, c.nu1)], d(Xh[24 * h:24 * h + 24]),
                              d(e)):
                inside = h
        if inside >= 0:
            E = Xh[24 * inside:24 * inside + 24]
            x = p - c.centers[inside]
            for r in range(6):
                e[r] -= E[r] + E[6 + 3 * r:9 + 3 * r] @ x
        tr = e[0] + e[3] + e[5]
        Sh[i] = c.sig_inf + 2 * mu0 * e + lam0 * tr * np.array([1, 0, 0, 1, 0, 1])
    assert scaled_err(S, Sh) < tol


def test_mixed_field_matches_fp64_field_far_and_near(g):
    """The mixed form's FP32 far path: a grid over a cube much wider than the
    microstructure, so that both paths run, against the FP64 sums (mixed-form tolerance;
    at the points farthest out every contribution takes the FP32 path)."""
    from ibemproject_gb300 import cases
    c = cases.ellipsoid_case(60, vf=0.1, seed=11)
    L = float(c.title.split("=")[1])
    pts = cases.cell_grid(12, -2.0 * L, 3.0 * L)
    rng = np.random.default_rng(2)
    E = rng.normal(size=24 * c.num) * 1e-3
    E[np.arange(c.num * 24) % 24 >= 6] /= 0.008   # gradient coefficients scale with 1 / length
    m = g.material(c.E0, c.nu0, c.E1, c.nu1)
    cen, ax, qt, Et, pt = dev(c.centers), dev(c.axes), dev(c.quats), dev(E), dev(pts)
    out = []
    for form in (0, 1):
        S = torch.zeros((len(pts), 6), dtype=torch.float64, device="cuda")
        g.check(g.lib().ibem_e3d_ell_field(form, P(pt), len(pts), P(cen), P(ax), P(qt), c.num, ctypes.byref(m),
                                           P(Et), d(np.zeros(6)), P(S), None))
        torch.cuda.synchronize()
        out.append(S.cpu().numpy())
    assert scaled_err(out[1], out[0]) < 1e-8
    # the slices' partial sums are added in a fixed order: a second call is bit-identical
    S = torch.zeros((len(pts), 6), dtype=torch.float64, device="cuda")
    g.check(g.lib().ibem_e3d_ell_field(0, P(pt), len(pts), P(cen), P(ax), P(qt), c.num, ctypes.byref(m), P(Et),
                                       d(np.zeros(6)), P(S), None))
    torch.cuda.synchronize()
    assert np.array_equal(S.cpu().numpy(), out[0])


def test_mixed_and_fp64_agree_at_larger_size(g):
    """Size-independent property: 400 ellipsoids (N = 9,600), both forms agree and the mixed
    form reaches its backward-error tolerance."""
    from ibemproject_gb300 import cases
    c = cases.ellipsoid_case(400, vf=0.15, seed=5)
    X64, _, r64 = g.run_host_ell(c, form=g.SOLVE_FP64)
    Xm, _, rm = g.run_host_ell(c, form=g.SOLVE_MIXED_IR, tol=1e-13)
    assert rm.backward_error <= 1e-13
    assert scaled_err(Xm, X64) < 1e-9


def test_ellipsoid_entry_points_check_arguments(g):
    m = g.material(70e9, 0.3, 400e9, 0.2)
    assert g.lib().ibem_e3d_ell_pair_blocks(None, None, None, 3, ctypes.byref(m), None, 72, 0, 0, None) == \
        g.IBEM_ERR_ARG
    assert g.lib().ibem_e3d_ell_field(7, None, 1, None, None, None, 0, ctypes.byref(m), None, None, None, None) == \
        g.IBEM_ERR_ARG


@pytest.mark.parametrize("form", ["bj", "mixed"])
def test_ellipsoid_batches_dense_solve_and_effective_modulus(g, form):
    """A ragged batch of ellipsoid realisations (different materials) through
    ibem_e3d_batch_dense_solve (block-Jacobi GMRES and the mixed LU form) against the plain
    FP64 pipeline of each realisation, and the effective moduli against their definition:
    <e> = C0^-1 : sigma + sum_p (V_p / V) E_p, V_p = 4/3 pi a1 a2 a3."""
    from ibemproject_gb300 import batch as B
    from ibemproject_gb300 import cases
    cs = [cases.ellipsoid_case(n, vf=v, seed=20 + n, E1=70e9 * c, method="mc")
          for n, v, c in ((7, 0.2, 3.0), (40, 0.27, 12.0), (1, 0.05, 5.7))]
    bt = B.DeviceBatch(cs)
    assert bt.ellipsoids
    sig = np.array([0, 0, 0, 0, 0, 1.0])
    b = B.farfield_rhs(bt, sig)
    f = g.SOLVE_GMRES_BJ if form == "bj" else g.SOLVE_MIXED_IR
    x, reps = B.dense_batch_solve(bt, b, f, tol=1e-12)
    vols = np.array([float(c.title.split("=")[1]) ** 3 for c in cs])
    e_eff, eps = B.effective_modulus(bt, x, sig, volume=vols)
    x = x.cpu().numpy()
    for s, c in enumerate(cs):
        rows = bt.seg_rows(s)
        xd, _, _ = g.run_host_ell(c, form=g.SOLVE_FP64)
        assert scaled_err(x[rows], xd) < 1e-8
        E = xd.reshape(-1, 24)[:, :6]
        vp = 4 / 3 * np.pi * c.axes.prod(axis=1)
        mean_star = (vp[:, None] * E).sum(axis=0) / vols[s]
        e33 = sig[5] / c.E0 + mean_star[5]   # remote strain of sigma33 alone: sigma33 / E0
        assert abs(e_eff[s] - sig[5] / e33) <= 1e-9 * abs(e_eff[s])
    with pytest.raises(ValueError):
        B.solve(bt, b)
