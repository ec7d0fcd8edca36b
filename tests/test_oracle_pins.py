"""The oracle (CPU restatement) against the reference's own outputs.

Fixtures in tests/golden were produced by the reference's elastic-3D translation
units compiled from source (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import case_from_npz, golden, scaled_err

ORDERS = [("D40", 0, 0), ("D50", 1, 0), ("D60", 2, 0), ("D41", 0, 1), ("D51", 1, 1), ("D61", 2, 1),
          ("D42", 0, 2), ("D52", 1, 2), ("D62", 2, 2)]


def test_kat_eshelby_tensors(oracle_mod):
    z = golden("kat_reference.npz")
    m = oracle_mod.mat(*z["mat"])
    for name, o, nd in ORDERS:
        for t, p in enumerate(z["points"]):
            got = oracle_mod.D_tensor(o, nd, p[:3], p[3], m)
            assert scaled_err(got, z[name][t]) < 1e-12, (name, t)


def test_kat_green(oracle_mod):
    z = golden("kat_reference.npz")
    m = oracle_mod.mat(*z["mat"])
    for t, p in enumerate(z["points"]):
        for o in range(3):
            assert scaled_err(oracle_mod.IGreen(o, p[:3], p[3], m), z[f"IG{o}"][t]) < 1e-12
        for nd in range(1, 5):
            assert scaled_err(oracle_mod.Green(nd, p[:3], m), z[f"G{nd}"][t]) < 1e-12


def test_tiny_case_assembly_solve_post(oracle_mod):
    z = golden("tiny_reference.npz")
    c = case_from_npz(z)
    H, G = oracle_mod.assemble(c, 78)
    assert scaled_err(H, z["HMAT"]) < 1e-12
    assert scaled_err(G, z["GMAT"]) < 1e-12
    A, b, tcol, t = oracle_mod.apply_bc(c, H, G)
    assert t == 3 * c.NN
    assert scaled_err(b, z["b"]) < 1e-12
    X = oracle_mod.solve_fullpiv(A, b)
    n3 = 3 * c.NN
    assert scaled_err(X[n3:], z["X"][n3:]) < 1e-9
    assert scaled_err(X[:n3], z["X"][:n3]) < 1e-9
    U, T = oracle_mod.get_ut(c, tcol, X)
    S = oracle_mod.post(c, 78, U[n3:], U[:n3], T)
    assert scaled_err(S, z["stress"]) < 1e-9


def test_example_fixture_matches_ground_truth():
    """The reference, built here, reproduces its published 7-digit stresses."""
    z = golden("example_reference.npz")
    gt = z["ground_truth"]
    assert np.all(np.abs(z["stress"] - gt) <= 5e-7 * np.abs(gt) + 1e-9 * np.abs(gt).max())


def test_example_post_subset(oracle_mod):
    """Oracle post-processing of the reference example (8 of 103 points) from the
    reference's own displacement/traction/eigenstrain solution."""
    z = golden("example_reference.npz")
    c = case_from_npz(z)
    n3 = 3 * c.NN
    idx = np.array([0, 13, 27, 40, 55, 70, 88, 102])
    S = oracle_mod.post(c, 78, z["U"][n3:], z["U"][:n3], z["T"], points=c.points[idx])
    assert scaled_err(S, z["stress"][idx]) < 1e-11
    gt = z["ground_truth"][idx]
    assert np.all(np.abs(S - gt) <= 5e-7 * np.abs(gt) + 1e-9 * np.abs(z["ground_truth"]).max())


def test_farfield_single_sphere_eshelby(oracle_mod):
    """Boundary-free loading (no reference counterpart): one sphere under a remote
    stress must give Eshelby's uniform equivalent eigenstrain,
    (C0 - C1) (eps_inf + S E) = C0 E,  S the interior Eshelby tensor of a sphere."""
    E0, nu0, E1, nu1 = 70e9, 0.3, 400e9, 0.2
    m = oracle_mod.mat(E0, nu0, E1, nu1)
    sig = np.array([0.3, 0.1, 0.0, -0.2, 0.05, 1.0])
    A = oracle_mod.pair_blocks(np.zeros((1, 3)), np.array([0.05]), m, 24)
    b = oracle_mod.farfield_rhs(1, m, 24, sig)
    X = np.linalg.solve(A, b)
    # closed form with 6x6 Voigt-like algebra over the i<=j unknowns
    pairs = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]

    def iso(lam, mu):
        C = np.zeros((3, 3, 3, 3))
        for i in range(3):
            for j in range(3):
                for k in range(3):
                    for l in range(3):
                        C[i, j, k, l] = lam * (i == j) * (k == l) + mu * ((i == k) * (j == l) + (i == l) * (j == k))
        return C
    mu0, mu1 = E0 / (2 * (1 + nu0)), E1 / (2 * (1 + nu1))
    C0 = iso(2 * mu0 * nu0 / (1 - 2 * nu0), mu0)
    C1 = iso(2 * mu1 * nu1 / (1 - 2 * nu1), mu1)
    S = np.zeros((3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    S[i, j, k, l] = ((5 * nu0 - 1) * (i == j) * (k == l)
                                     + (4 - 5 * nu0) * ((i == k) * (j == l) + (i == l) * (j == k))) / (15 * (1 - nu0))
    Sg = np.array([[sig[0], sig[1], sig[2]], [sig[1], sig[3], sig[4]], [sig[2], sig[4], sig[5]]])
    eps = ((1 + nu0) * Sg - nu0 * np.trace(Sg) * np.eye(3)) / E0
    dC = C0 - C1
    M = np.einsum("ijkl,klmn->ijmn", dC, S) - C0
    rhs = -np.einsum("ijkl,kl->ij", dC, eps)
    # 9x9 system is singular on antisymmetric tensors; the minimum-norm solution is the symmetric one
    Em = np.linalg.lstsq(M.reshape(9, 9), rhs.reshape(9), rcond=None)[0].reshape(3, 3)
    want = np.array([Em[i, j] for (i, j) in pairs])
    assert scaled_err(X[:6], want) < 1e-12
    assert np.abs(X[6:]).max() < 1e-12 * np.abs(want).max()
