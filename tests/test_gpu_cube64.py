"""The bounded-cube workload end to end on the GPU against the reference itself.

Unit cube, 6 x 10 x 10 Q4 boundary elements (600 elements, 602 nodes), bottom face fixed,
unit normal traction on the top face, 64 spheres of radius 0.05 placed by random
sequential addition (seed 12345, centre distance >= 2.2 r), E0 = 70 GPa / nu0 = 0.3,
E1 = 400 GPa / nu1 = 0.2.  The fixture (tests/golden/make_golden.py cube64) holds the
reference's own solution X (78 unknowns per sphere, N = 6,798: its assembly, ApplyBC and
Eigen fullPivLu) and its stresses at a seeded 1,024-point subset of the 32^3 cell-centred
grid, plus the oracle's solution of the 24-unknown truncation (N = 3,342).

Tolerances (relative to the largest entry): eigenstrain coefficients and stresses 1e-9
for the plain FP64 form, 1e-8 for the mixed form (FP32 LU + FP64 GMRES-IR).
"""
import numpy as np
import pytest

from conftest import golden, scaled_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g():
    import ibemproject_gb300 as g
    g.lib()
    return g


@pytest.fixture(scope="module")
def cube():
    from ibemproject_gb300 import cases
    z = golden("cube64_reference.npz")
    c = cases.bounded_cube_case(n_face=10, num=64, radius=0.05, grid=0, seed=12345)
    assert np.array_equal(c.centers, z["centers"]) and np.array_equal(c.radius, z["radius"])
    c.points = z["points"]
    return z, c


def _orders(X, n3, layout):
    """Eigenstrain coefficients by order: (order 0, order 1[, order 2]) across spheres."""
    E = X[n3:].reshape(-1, layout)
    return [E[:, :6], E[:, 6:24]] + ([E[:, 24:]] if layout > 24 else [])


@pytest.mark.parametrize("layout,form,tol", [(78, 0, 1e-9), (78, 1, 1e-8), (24, 0, 1e-9), (24, 1, 1e-8)])
def test_bounded_cube_64_spheres(g, cube, layout, form, tol):
    z, c = cube
    X, S, rep = g.run_host(c, layout=layout, form=form, tol=1e-14)
    n3 = 3 * c.NN
    Xr, Sr = (z["X78"], z["stress78"]) if layout == 78 else (z["X24"], z["stress24"])
    assert len(X) == len(Xr) == n3 + layout * c.num
    # every order of the eigenstrain on its own scale, the boundary unknowns, the stresses
    for got, want in zip(_orders(X, n3, layout), _orders(Xr, n3, layout)):
        assert scaled_err(got, want) < tol
    assert scaled_err(X[:n3], Xr[:n3]) < tol
    assert scaled_err(S, Sr) < tol
