"""The generated sphere / boundary code (ibemproject_gb300/csrc/gen_*.cuh), compiled for
the host, against the oracle: same straight-line source the GPU kernels inline."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, scaled_err

HG = os.path.join(ROOT, "tests", "hostgen")
SO = os.path.join(HG, "_build", "libhostgen.so")
MAT = (70e9, 0.3, 400e9, 0.2)


@pytest.fixture(scope="module")
def hg():
    from ibemproject_gb300 import codegen
    codegen.generate()
    os.makedirs(os.path.dirname(SO), exist_ok=True)
    subprocess.run(["g++", "-O0", "-shared", "-fPIC", "-I", os.path.join(ROOT, "ibemproject_gb300", "csrc"),
                    "-o", SO, os.path.join(HG, "hostgen.cpp")], check=True)
    return ctypes.CDLL(SO)


_dp = ctypes.POINTER(ctypes.c_double)


def d(a):
    return a.ctypes.data_as(_dp)


def _mat():
    return [ctypes.c_double(v) for v in MAT]


@pytest.mark.parametrize("layout", [24, 60, 78])
def test_pair_blocks(hg, oracle_mod, layout):
    m = oracle_mod.mat(*MAT)
    cen = np.array([[0.5, 0.5, 0.5], [0.61, 0.47, 0.52], [0.41, 0.58, 0.44]])
    rad = np.array([0.05, 0.04, 0.045])
    A = oracle_mod.pair_blocks(cen, rad, m, layout)
    nu = layout
    for s in range(3):
        for h in range(3):
            x = np.ascontiguousarray(cen[s] - cen[h])
            out = np.zeros(nu * nu)
            hg.hg_pair_block(layout, d(x), ctypes.c_double(rad[h]), *_mat(), int(s == h), d(out))
            assert scaled_err(out.reshape(nu, nu), A[nu * s:nu * s + nu, nu * h:nu * h + nu]) < 1e-13


@pytest.mark.parametrize("layout", [24, 60, 78])
def test_node_and_field(hg, oracle_mod, layout):
    m = oracle_mod.mat(*MAT)
    rng = np.random.default_rng(11)
    for t in range(4):
        x = rng.normal(size=3) * 0.2
        a = 0.05
        out = np.zeros(3 * layout)
        hg.hg_node(layout, d(x), ctypes.c_double(a), *_mat(), d(out))
        H = np.zeros((3, layout), order="F")
        oracle_mod.lib().orc_node_blocks(1, d(np.ascontiguousarray(x)), 1, d(np.zeros(3)), d(np.array([a])),
                                         ctypes.byref(m), layout, d(H), 3, 0, 0)
        assert scaled_err(out.reshape(3, layout), H) < 1e-13
    # field: one particle, points outside and inside, against the oracle's post
    from ibemproject_gb300.cases import Case
    E = rng.normal(size=layout)
    pts = np.array([[0.13, -0.05, 0.02], [0.01, 0.02, -0.015], [0.0, 0.0, 0.0]])
    c = Case(*MAT, np.zeros((0, 3)), np.zeros((0, 4), np.int32), np.zeros((0, 2)), np.zeros((0, 24)),
             np.zeros((1, 3)), np.array([0.05]), pts)
    want = oracle_mod.post(c, layout, E, sig_inf=np.zeros(6))
    mu0 = MAT[0] / (2 * (1 + MAT[1]))
    lam0 = 2 * mu0 * MAT[1] / (1 - 2 * MAT[1])
    for k, p in enumerate(pts):
        e = np.zeros(6)
        hg.hg_field(layout, d(np.ascontiguousarray(p)), ctypes.c_double(0.05), *_mat(), d(E), d(e))
        if p @ p <= 0.05 ** 2:   # local eigenstrain subtraction is done by the kernel wrapper
            x = p
            loc = E[:6].copy()
            for r in range(6):
                loc[r] += E[6 + 3 * r:9 + 3 * r] @ x
                if layout == 78:
                    M = E[24 + 9 * r:33 + 9 * r].reshape(3, 3)
                    loc[r] += sum((1 if i == j else 2) * M[i, j] * x[i] * x[j] for i in range(3) for j in range(i, 3))
                elif layout == 60:
                    v = E[24 + 6 * r:30 + 6 * r]
                    pr = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
                    loc[r] += sum((1 if i == j else 2) * v[t] * x[i] * x[j] for t, (i, j) in enumerate(pr))
            e -= loc
        tr = e[0] + e[3] + e[5]
        s = np.array([lam0 * tr + 2 * mu0 * e[0], 2 * mu0 * e[1], 2 * mu0 * e[2],
                      lam0 * tr + 2 * mu0 * e[3], 2 * mu0 * e[4], lam0 * tr + 2 * mu0 * e[5]])
        assert scaled_err(s, want[k]) < 1e-13


@pytest.mark.parametrize("order", [0, 1, 2])
def test_bem_stress_kernels(hg, oracle_mod, order):
    m = oracle_mod.mat(*MAT)
    mu0 = MAT[0] / 2.6
    lam0 = 2 * mu0 * 0.3 / 0.4
    mu1 = MAT[2] / 2.4
    lam1 = 2 * mu1 * 0.2 / 0.6
    rng = np.random.default_rng(5 + order)
    for t in range(4):
        x = rng.normal(size=3) * 0.3
        nv = rng.normal(size=3)
        nv /= np.linalg.norm(nv)
        nrow = 6 * 3 ** order
        su = np.zeros(nrow * 3)
        st = np.zeros(nrow * 3)
        hg.hg_bem_stress(order, d(x), d(nv), *_mat(), ctypes.c_double(lam0 - lam1), ctypes.c_double(mu0 - mu1),
                         d(su), d(st))
        rsu, rst = oracle_mod.stress_kernel(x, nv, m, lam0 - lam1, mu0 - mu1, order)
        assert scaled_err(su.reshape(nrow, 3), rsu) < 1e-13
        assert scaled_err(st.reshape(nrow, 3), rst) < 1e-13


def test_contracted_field_matches_generated(hg):
    """The hand-contracted field sum (csrc/field_contract.cuh) equals the generated
    entry-by-entry sum, outside, near and inside the sphere."""
    rng = np.random.default_rng(17)
    for t in range(40):
        x = rng.normal(size=3) * (0.03 if t % 4 == 0 else 0.15)
        a = 0.05
        E = rng.normal(size=24)
        e1 = np.zeros(6)
        e2 = np.zeros(6)
        hg.hg_field(24, d(x), ctypes.c_double(a), *_mat(), d(E), d(e1))
        hg.hg_field24c(d(x), ctypes.c_double(a), *_mat(), d(E), d(e2))
        assert scaled_err(e2, e1) < 1e-13, (t, x, e1, e2)


def test_layout60_fp32_column_groups_match_fp64_blocks(hg):
    """The FP32 column groups of the layout-60 blocks (the matrix-free solver's GMRES product,
    gen_sphere60_f32.cuh) cover every entry of the FP64 pair block exactly once: each
    (row order, column order) sub-block within 2e-5 of its largest entry, outside and inside
    the unit source sphere."""
    rng = np.random.default_rng(41)
    for k in range(12):
        x = rng.normal(size=3)
        x *= (0.5 if k % 4 == 0 else rng.uniform(2.1, 12.0)) / np.linalg.norm(x)
        o64, o32 = np.zeros(3600), np.zeros(3600)
        hg.hg_block60_groups(d(x), *_mat(), d(o64), d(o32))
        B64, B32 = o64.reshape(60, 60), o32.reshape(60, 60)
        edges = (0, 6, 24, 60)
        for ro in range(3):
            for co in range(3):
                rs, cs = slice(edges[ro], edges[ro + 1]), slice(edges[co], edges[co + 1])
                m = np.abs(B64[rs, cs]).max()
                if m == 0.0:   # some sub-blocks vanish inside the sphere
                    assert np.abs(B32[rs, cs]).max() <= 1e-6 * np.abs(B64).max(), (k, ro, co)
                    continue
                assert np.abs(B32[rs, cs] - B64[rs, cs]).max() <= 2e-5 * m, (k, ro, co)


def test_bem_post_contracted_matches_generated(hg):
    """The boundary part of the stresses contracted with the boundary displacement and traction
    before forming any tensor (bem_contract.cuh) against the generated Kelvin kernels
    (bem_stress_post) contracted afterwards: 1e-13 of the largest component, Gauss points from
    0.01 to 100 units away, two materials."""
    rng = np.random.default_rng(31)
    for k in range(200):
        x = rng.normal(size=3) * 10.0 ** rng.uniform(-2, 2)
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        u, t = rng.normal(size=3), rng.normal(size=3) * 1e9
        mat = (70e9, 0.3, 400e9, 0.2) if k % 2 else (210e9, 0.27, 70e9, 0.35)
        sc, sg = np.zeros(6), np.zeros(6)
        hg.hg_bem_post_pair(d(x), d(n), d(u), d(t), *[ctypes.c_double(v) for v in mat], d(sc), d(sg))
        assert np.abs(sc - sg).max() <= 1e-13 * np.abs(sg).max(), (k, sc, sg)


def test_bem_post_double_float_matches_fp64(hg):
    """The mixed form's double-float boundary contraction (compensated sums on the FP32 pipe)
    against the FP64 one: 1e-12 of the largest component, Gauss points 0.01 to 10 units from
    sample points in a unit-scale box, weights and tractions of realistic size."""
    rng = np.random.default_rng(37)
    worst = 0.0
    for k in range(300):
        p = rng.uniform(0, 1, size=3)
        x = rng.normal(size=3) * 10.0 ** rng.uniform(-2, 1)
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        rec = np.concatenate([p + x, n, [rng.uniform(1e-4, 1e-2)], rng.normal(size=3) * 1e-11, rng.normal(size=3)])
        sd, sf = np.zeros(6), np.zeros(6)
        hg.hg_bem_post_pair_df(d(p), d(rec), *[ctypes.c_double(v) for v in (70e9, 0.3, 400e9, 0.2)], d(sd), d(sf))
        worst = max(worst, np.abs(sd - sf).max() / np.abs(sf).max())
    assert worst < 3e-12, worst


def test_double_float_field_matches_fp64(hg):
    """The double-float contraction (csrc/field_contract.cuh, mixed form) agrees with the
    FP64 one to ~1e-12 of the strain, for spheres from micro- to metre-sized (the scaled
    coordinates keep FP32's exponent range), outside, near and inside."""
    rng = np.random.default_rng(23)
    for t in range(60):
        a = 10.0 ** rng.uniform(-5, 2)
        cen = rng.normal(size=3) * a * 30
        x = rng.normal(size=3) * a * (0.6 if t % 5 == 0 else rng.uniform(1.2, 40))
        E = rng.normal(size=24)
        E[6:] /= a   # order-1 eigenstrain per unit length
        e1 = np.zeros(6)
        e2 = np.zeros(6)
        hg.hg_field24c(d(x), ctypes.c_double(a), *_mat(), d(E), d(e1))
        hg.hg_field24df(d(cen + x), d(cen), ctypes.c_double(a), *_mat(), d(E), d(e2))
        assert scaled_err(e2, e1) < 2e-12, (t, a, x, e1, e2)


@pytest.mark.parametrize("fp32", [0, 1])
def test_pair_apply_matches_generated_block(hg, fp32):
    """The matrix-free pair product (mf_contract.cuh: contracted strain and its analytic
    gradient) against the generated 24 x 24 block times the same coefficients, outside and
    inside the source sphere.  FP64 to 1e-12; FP32 (unit source radius, as the solver
    calls it) to 2e-5 of the largest entry."""
    rng = np.random.default_rng(5)
    for t in range(40):
        a = 1.0 if fp32 else 0.05 * (0.8 + 0.4 * rng.random())
        if t < 4:
            x = rng.normal(size=3) * 0.3 * a       # inside
        else:
            x = rng.normal(size=3)
            x *= a * (1.02 + 6 * rng.random()) / np.linalg.norm(x)
        coef = rng.normal(size=24)
        coef[6:] /= a
        blk = np.zeros(24 * 24)
        hg.hg_pair_block(24, d(np.ascontiguousarray(x)), ctypes.c_double(a), *_mat(), 0, d(blk))
        want = blk.reshape(24, 24) @ coef
        got = np.zeros(24)
        hg.hg_pair_apply24(fp32, d(np.ascontiguousarray(x)), ctypes.c_double(a), *_mat(), d(coef), d(got))
        tol = 2e-5 if fp32 else 1e-12
        assert np.abs(got[:6] - want[:6]).max() <= tol * np.abs(want[:6]).max(), (t, got[:6], want[:6])
        assert np.abs(got[6:] - want[6:]).max() <= tol * np.abs(want[6:]).max(), (t, got[6:], want[6:])


def test_field24_f32_far_pairs(hg):
    """The FP32 far-pair contraction of the mixed stress sums against the FP64 contraction:
    beyond 12 radii (the split's threshold) its relative error stays at the FP32 rounding
    level (< 3e-6 of the largest strain component), and its size relative to a
    contact-distance sphere is below (1/12)^3, which is what bounds its share of the summed
    error."""
    rng = np.random.default_rng(21)
    worst = 0.0
    for t in range(200):
        a = 0.012 * (0.8 + 0.4 * rng.random())
        cen = rng.random(3) * 0.4
        x = rng.normal(size=3)
        x *= a * (12.0 + 30.0 * rng.random()) / np.linalg.norm(x)
        E = rng.normal(size=24) * 1e-3
        E[6:] /= a
        e1, e2 = np.zeros(6), np.zeros(6)
        hg.hg_field24c(d(np.ascontiguousarray(x)), ctypes.c_double(a), *_mat(), d(E), d(e1))
        hg.hg_field24f32(d(cen + x), d(cen), ctypes.c_double(a), *_mat(), d(E), d(e2))
        worst = max(worst, scaled_err(e2, e1))
    assert worst < 3e-6, worst
