"""Whole pipeline through the host-buffer C ABI (ibem_e3d_run_host / run_dir) on GPU,
against the reference's outputs and the oracle.  Tolerances: 1e-9 of the largest entry
on eigenstrain coefficients and stresses (plain FP64 form); 1e-8 for the mixed form."""
import os
import tempfile

import numpy as np
import pytest

from conftest import case_from_npz, golden, scaled_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import ibemproject_gb300 as g
    g.lib()
    return g


def test_reference_example_end_to_end(g):
    """examples/elastic3D_spherical: 1176 Q4 elements, 2 spheres, 78 unknowns/particle."""
    z = golden("example_reference.npz")
    c = case_from_npz(z)
    X, S, rep = g.run_host(c, layout=78, form=g.SOLVE_FP64)
    n3 = 3 * c.NN
    assert scaled_err(X[n3:], z["X"][n3:]) < 1e-9
    assert scaled_err(S, z["stress"]) < 1e-9
    gt = z["ground_truth"]
    assert np.all(np.abs(S - gt) <= 5e-7 * np.abs(gt) + 1e-9 * np.abs(gt).max())


def test_reference_example_mixed_form(g):
    z = golden("example_reference.npz")
    c = case_from_npz(z)
    X, S, rep = g.run_host(c, layout=78, form=g.SOLVE_MIXED_IR, tol=1e-14)
    n3 = 3 * c.NN
    assert scaled_err(X[n3:], z["X"][n3:]) < 1e-8
    assert scaled_err(S, z["stress"]) < 1e-8


def test_run_dir_reads_reference_files(g):
    from ibemproject_gb300 import cases
    z = golden("tiny_reference.npz")
    c = case_from_npz(z)
    with tempfile.TemporaryDirectory() as d:
        cases.write_case(d, c)
        rep = g.run_dir(d, layout=78)
        S = np.loadtxt(os.path.join(d, "stress.txt"))
    # stress.txt holds 7 significant digits, as the reference writes it
    assert np.all(np.abs(S - z["stress"]) <= 1e-6 * np.abs(z["stress"]).max())


def test_run_dir_from_side_car_matches_text(g):
    """ibem_e3d_run_dir on the binary side-car (case.ibemb) writes the same stress.txt as on
    the text files it was made from."""
    from ibemproject_gb300 import cases
    z = golden("tiny_reference.npz")
    c = case_from_npz(z)
    with tempfile.TemporaryDirectory() as d:
        cases.write_case(d, c)
        g.run_dir(d, layout=78)
        text = open(os.path.join(d, "stress.txt")).read()
        g.sidecar_from_txt(d)
        for f in ("position.txt", "BEM.txt", "postprocess.txt"):
            os.remove(os.path.join(d, f))
        assert g.read_case_native(d)[1]
        g.run_dir(d, layout=78)
        assert open(os.path.join(d, "stress.txt")).read() == text


@pytest.mark.parametrize("layout", [24, 60])
def test_truncated_layouts_vs_oracle(g, oracle_mod, layout):
    """Layouts without a reference counterpart: the same entries, truncated (24) or with
    the order-2 coefficients stored once per symmetric pair (60), solved by the oracle."""
    from ibemproject_gb300 import cases
    c = cases.bounded_cube_case(n_face=3, num=4, radius=0.08, grid=4, seed=3, top_traction=1e4)
    X, S, rep = g.run_host(c, layout=layout)
    H, G = oracle_mod.assemble(c, layout)
    A, b, tcol, t = oracle_mod.apply_bc(c, H, G)
    Xo = oracle_mod.solve_fullpiv(A, b)
    n3 = 3 * c.NN
    assert scaled_err(X[n3:], Xo[n3:]) < 1e-9
    U, T = oracle_mod.get_ut(c, tcol, Xo)
    So = oracle_mod.post(c, layout, U[n3:], U[:n3], T)
    assert scaled_err(S, So) < 1e-9


@pytest.mark.parametrize("form", [0, 1])
def test_farfield_case_vs_oracle(g, oracle_mod, form):
    from ibemproject_gb300 import cases
    c = cases.farfield_case(num=60, r0=0.05, vf=0.12, grid=5, seed=9)
    X, S, rep = g.run_host(c, layout=24, form=form, tol=1e-14)
    m = oracle_mod.case_mat(c)
    A = oracle_mod.pair_blocks(c.centers, c.radius, m, 24)
    b = oracle_mod.farfield_rhs(c.num, m, 24, c.sig_inf)
    Xo = np.linalg.solve(A, b)
    assert scaled_err(X, Xo) < (1e-9 if form == 0 else 1e-8)
    So = oracle_mod.post(c, 24, Xo, sig_inf=c.sig_inf)
    assert scaled_err(S, So) < (1e-9 if form == 0 else 1e-8)


def test_mixed_matches_fp64_at_scale(g):
    """Size-independent property at a larger size: both forms agree and the mixed
    form's FP64 backward error reaches the tolerance."""
    from ibemproject_gb300 import cases
    c = cases.farfield_case(num=400, r0=0.012, vf=0.15, grid=0, seed=21)
    X64, _, r64 = g.run_host(c, layout=24, form=g.SOLVE_FP64)
    Xm, _, rm = g.run_host(c, layout=24, form=g.SOLVE_MIXED_IR, tol=1e-13)
    assert rm.backward_error <= 1e-13
    assert scaled_err(Xm, X64) < 1e-9
