"""Ellipsoidal inclusions without a GPU: the library's evaluator (csrc/ellipsoid.cuh, the
same source the CUDA kernels inline) compiled for the host, against

* the reference's sphere tensors in the sphere limit (the oracle's D tensors and pair
  blocks, themselves pinned to the reference: tests/test_oracle_pins.py), any rotation;
* an evaluation that shares nothing with it: volume quadrature of the differentiated
  kernels over the ellipsoid (oracle/ell_oracle.c), at exterior points, orders 0/1 of the
  eigenstrain, strain and strain gradient;
* Eshelby's interior tensor of an ellipsoid in the closed form of T. Mura,
  Micromechanics of Defects in Solids (1987), eq. 11.16 / 11.22, with the integrals I_i,
  I_ij computed by quadrature;
* the reference's spheroid formulas (integratorhelperPotential3D_elliptical.cpp:11-26
  depolarisation integral, :650-654 lambda), restated here in numpy;
* Carlson's R_F / R_D (scalar, oracle/ell_oracle.c) and a quadrature of every I_k.
Tolerances: 1e-12 (closed forms, sphere limit), 1e-11 (quadrature, exterior)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, scaled_err

HG = os.path.join(ROOT, "tests", "hostgen")
SO = os.path.join(HG, "_build", "libhostell.so")
MAT = (70e9, 0.3, 400e9, 0.2)
_dp = ctypes.POINTER(ctypes.c_double)


def d(a):
    return np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(_dp)


@pytest.fixture(scope="module")
def he():
    os.makedirs(os.path.dirname(SO), exist_ok=True)
    subprocess.run(["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-I",
                    os.path.join(ROOT, "ibemproject_gb300", "csrc"), "-o", SO, os.path.join(HG, "hostell.cpp")],
                   check=True)
    L = ctypes.CDLL(SO)
    L.he_lambda.restype = ctypes.c_double
    return L


def rot(he, q):
    Q = np.zeros(9)
    he.he_rot(d(np.asarray(q, dtype=np.float64)), d(Q))
    return Q.reshape(3, 3)


def D_lib(he, order, nder, x, q, a, nu=MAT[1]):
    out = np.zeros(3 ** (4 + order + nder))
    he.he_D(order, nder, d(x), d(q), d(a), ctypes.c_double(nu), d(out))
    return out.reshape((3,) * (4 + order + nder))


def multi_indices():
    ks = []
    for deg in range(4):
        for k1 in range(deg, -1, -1):
            for k2 in range(deg - k1, -1, -1):
                ks.append((k1, k2, deg - k1 - k2))
    return ks


Q_RAND = np.array([0.9, 0.1, -0.3, 0.2])


def test_sphere_limit_blocks_match_reference_spheres(he, oracle_mod):
    m = oracle_mod.mat(*MAT)
    cen = np.array([[0.5, 0.5, 0.5], [0.61, 0.47, 0.52], [0.41, 0.58, 0.44]])
    rad = np.array([0.05, 0.04, 0.045])
    A = oracle_mod.pair_blocks(cen, rad, m, 24)
    for s in range(3):
        for h in range(3):
            out = np.zeros(576)
            he.he_block24(d(cen[s] - cen[h]), d(Q_RAND), d(np.full(3, rad[h])), *[ctypes.c_double(v) for v in MAT],
                          int(s == h), d(out))
            assert scaled_err(out.reshape(24, 24), A[24 * s:24 * s + 24, 24 * h:24 * h + 24]) < 1e-12


@pytest.mark.parametrize("order,nder", [(0, 0), (0, 1), (1, 0), (1, 1)])
def test_sphere_limit_D_tensors(he, oracle_mod, order, nder):
    m = oracle_mod.mat(*MAT)
    for x in ([0.071, -0.032, 0.055], [0.0301, 0.0402, 0.0], [0.012, -0.02, 0.015]):
        want = oracle_mod.D_tensor(order, nder, np.array(x), 0.05, m)
        got = D_lib(he, order, nder, np.array(x), Q_RAND, np.full(3, 0.05))
        assert scaled_err(got, want) < 1e-12


@pytest.mark.parametrize("order,nder", [(0, 0), (0, 1), (1, 0), (1, 1)])
@pytest.mark.parametrize("dist", [1.6, 3.0])
def test_exterior_vs_volume_quadrature(he, oracle_mod, order, nder, dist):
    """Exterior points at 1.6 and 3 times the longest semi-axis from the centre, along a
    direction oblique to every principal axis; aspect ratios 1 : 0.7 : 0.4."""
    a = np.array([0.01, 0.007, 0.004])
    Q = rot(he, Q_RAND / np.linalg.norm(Q_RAND))
    u = np.array([0.6, 0.5, 0.55])
    x = Q @ (u / np.linalg.norm(u) * dist * a[0])
    want = oracle_mod.ell_D_quad(order, nder, x, a, Q, MAT[1], n=(40, 40, 80))
    assert scaled_err(D_lib(he, order, nder, x, Q_RAND, a), want) < 1e-11


def test_interior_eshelby_tensor_matches_closed_form(he, oracle_mod):
    """Uniform eigenstrain, any interior point: D = Eshelby's S (principal frame)."""
    nu = MAT[1]
    a = np.array([0.01, 0.007, 0.004])
    abc = a.prod()
    Ii = [2 * np.pi * abc * oracle_mod.ell_I([int(i == m) for i in range(3)], a, 0.0, 200) for m in range(3)]
    Iij = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            k = [0, 0, 0]
            k[i] += 1
            k[j] += 1
            Iij[i, j] = 2 * np.pi * abc * oracle_mod.ell_I(k, a, 0.0, 200)
    c = 1 / (8 * np.pi * (1 - nu))
    S = np.zeros((3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            if i == j:
                S[i, i, i, i] = 3 * c * a[i] ** 2 * Iij[i, i] + (1 - 2 * nu) * c * Ii[i]
            else:
                S[i, i, j, j] = c * a[j] ** 2 * Iij[i, j] - (1 - 2 * nu) * c * Ii[i]
                v = (a[i] ** 2 + a[j] ** 2) / (16 * np.pi * (1 - nu)) * Iij[i, j] + \
                    (1 - 2 * nu) / (16 * np.pi * (1 - nu)) * (Ii[i] + Ii[j])
                S[i, j, i, j] = S[i, j, j, i] = S[j, i, i, j] = S[j, i, j, i] = v
    for x in (np.zeros(3), np.array([0.002, -0.001, 0.0005])):
        assert scaled_err(D_lib(he, 0, 0, x, [1.0, 0, 0, 0], a), S) < 1e-12


def test_gradient_rows_are_the_derivative_of_the_strain_rows(he):
    """Order-1 rows (the strain gradient at the collocation centre) against central
    differences of the order-0 rows, inside and outside."""
    a = np.array([0.01, 0.007, 0.004])
    for x, tol in ((np.array([0.002, -0.001, 0.0005]), 1e-9), (np.array([0.012, 0.004, 0.003]), 1e-6)):
        G = D_lib(he, 1, 1, x, Q_RAND, a)
        fd = np.zeros_like(G)
        h = 1e-6
        for r in range(3):
            e = np.zeros(3)
            e[r] = h
            fd[..., r] = (D_lib(he, 1, 0, x + e, Q_RAND, a) - D_lib(he, 1, 0, x - e, Q_RAND, a)) / (2 * h)
        assert scaled_err(G, fd) < tol


@pytest.mark.parametrize("lam", [0.0, 2e-5, 1e-3])
def test_depolarisation_integrals(he, oracle_mod, lam):
    a = np.array([0.01, 0.007, 0.004])
    x = a ** 2 + lam
    ik = np.zeros(20)
    he.he_ik(d(x), d(ik))
    for i, k in enumerate(multi_indices()):
        want = oracle_mod.ell_I(k, a, lam, 200)
        assert abs(ik[i] - want) <= 1e-12 * abs(want)
    assert abs(ik[0] - 2 * oracle_mod.carlson_rf(*x)) <= 1e-14 * ik[0]
    for m in range(3):   # I_{e_m} = 2/3 R_D with the distinguished argument last
        o = [x[(m + 1) % 3], x[(m + 2) % 3], x[m]]
        e = np.zeros(3, int)
        e[m] = 1
        want = 2 / 3 * oracle_mod.carlson_rd(*o)
        assert abs(ik[multi_indices().index(tuple(e))] - want) <= 1e-14 * want
    # sum_m I_{e_m} = 2 / Delta(lambda)
    assert abs(ik[1] + ik[2] + ik[3] - 2 / np.sqrt(np.prod(x))) <= 1e-13 * (ik[1] + ik[2] + ik[3])


def test_spheroid_forms_of_the_reference(he):
    """Prolate and oblate spheroids against the reference's closed forms of lambda
    (integratorhelperPotential3D_elliptical.cpp:650-654) and of the depolarisation
    integral I = 2 pi a1 a2 a3 int_lambda^inf ds / Delta (:11-26, restated)."""
    rng = np.random.default_rng(5)
    for a in (np.array([0.01, 0.004, 0.004]), np.array([0.004, 0.01, 0.01])):
        orient = 0   # the distinct axis
        a_u, a_e = a[orient], a[(orient + 1) % 3]
        a_l, a_s = a.max(), a.min()
        for _ in range(6):
            y = rng.normal(size=3) * 0.02
            if (y ** 2 / a ** 2).sum() <= 1:
                continue
            r2 = (y ** 2).sum()
            lam_ref = 0.5 * (r2 - a_u ** 2 - a_e ** 2 + np.sqrt((r2 + a_u ** 2 - a_e ** 2) ** 2
                                                                - 4 * (a_u ** 2 - a_e ** 2) * y[orient] ** 2))
            lam = he.he_lambda(d(y), d(a ** 2))
            assert abs(lam - lam_ref) <= 1e-12 * lam_ref
            b_bar = np.sqrt((a_u ** 2 + lam) / (a_e ** 2 + lam))
            val = np.arccosh(b_bar) if a_u > a_e else np.arccos(b_bar)
            I_ref = 4 * np.pi * a_u * a_e * a_e * val / np.sqrt(a_l ** 2 - a_s ** 2)
            ik = np.zeros(20)
            he.he_ik(d(a ** 2 + lam), d(ik))
            assert abs(2 * np.pi * a.prod() * ik[0] - I_ref) <= 1e-12 * I_ref


def test_rotation_is_a_change_of_frame(he):
    """Rotating the ellipsoid and the evaluation point together rotates every index of D."""
    a = np.array([0.01, 0.007, 0.004])
    x_loc = np.array([0.011, 0.006, -0.004])
    D0 = D_lib(he, 1, 1, x_loc, [1.0, 0, 0, 0], a)
    Q = rot(he, Q_RAND / np.linalg.norm(Q_RAND))
    D1 = D_lib(he, 1, 1, Q @ x_loc, Q_RAND, a)
    want = np.einsum("ia,jb,kc,ld,pe,rf,abcdef->ijklpr", Q, Q, Q, Q, Q, Q, D0)
    assert scaled_err(D1, want) < 1e-13


def test_single_precision_blocks(he):
    """The FP32 instantiation (the far-field path of the products) within 1e-5 of FP64."""
    a = np.array([0.01, 0.007, 0.004])
    x = np.array([0.05, -0.03, 0.02])
    o64, o32 = np.zeros(576), np.zeros(576)
    args = (d(x), d(Q_RAND), d(a), *[ctypes.c_double(v) for v in MAT], 0)
    he.he_block24(*args[:-1], 0, d(o64))
    he.he_block24_f32(*args[:-1], 0, d(o32))
    assert scaled_err(o32, o64) < 1e-5
