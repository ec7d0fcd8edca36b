"""The native microstructure generator (ibem_e3d_generate_spheres, host code of
libibem_gb300.so; no GPU): every pair keeps its minimum distance, radii and centres stay in
their ranges, the volume fraction is the one asked for, a seed names one microstructure, the
Monte Carlo method reaches 30% (where addition jams) without leaving a lattice behind, and an
unreachable packing is an error, not a hang."""
import ctypes

import numpy as np
import pytest


def gen(num, vf, seed=3, method="mc", r0=0.008):
    from ibemproject_gb300 import cases
    c = cases.generated_case(num, r0, vf, seed=seed, method=method)
    return c, float(c.title.split("=")[1])


def pair_ratio(C, R, gap=0.1):
    d = np.sqrt(((C[:, None] - C[None]) ** 2).sum(-1))
    m = R[:, None] + R[None] + gap * np.maximum(R[:, None], R[None])
    np.fill_diagonal(d, np.inf)
    return float((d / m).min())


@pytest.mark.parametrize("method,num,vf", [("rsa", 1, 0.1), ("rsa", 200, 0.15), ("rsa", 2000, 0.15),
                                           ("mc", 1, 0.2), ("mc", 50, 0.3), ("mc", 500, 0.3), ("mc", 1500, 0.25)])
def test_spheres_clear_every_pair_and_fill_the_volume(method, num, vf):
    r0 = 0.008
    c, L = gen(num, vf, method=method, r0=r0)
    C, R = c.centers, c.radius
    assert C.shape == (num, 3) and R.shape == (num,)
    assert R.min() >= 0.8 * r0 and R.max() <= 1.2 * r0
    if num > 1:
        assert pair_ratio(C, R) >= 1.0 - 1e-12
    vol = float(np.sum(4.0 / 3.0 * np.pi * R ** 3))
    assert abs(vol / L ** 3 - vf) <= 1e-12 * vf
    if method == "rsa":   # every sphere inside the cube
        assert (C - R[:, None]).min() >= 0 and (C + R[:, None]).max() <= L
    else:                 # centres in the cube
        assert C.min() >= 0 and C.max() <= L


def test_seed_names_one_microstructure():
    a, _ = gen(300, 0.25, seed=11)
    b, _ = gen(300, 0.25, seed=11)
    c, _ = gen(300, 0.25, seed=12)
    assert np.array_equal(a.centers, b.centers) and np.array_equal(a.radius, b.radius)
    assert not np.allclose(a.centers, c.centers)


def test_monte_carlo_leaves_no_lattice_behind():
    """Nearest-neighbour distances spread like a fluid's; no centre is left on a face."""
    c, L = gen(1000, 0.3, seed=5)
    C = c.centers
    d = np.sqrt(((C[:, None] - C[None]) ** 2).sum(-1))
    np.fill_diagonal(d, np.inf)
    nn = d.min(1)
    assert nn.std() / nn.mean() > 0.04
    assert np.sum((C == 0) | (C == L)) == 0
    # mean occupancy of the eight octants is uniform within sampling noise
    oct_ = ((C > L / 2) * np.array([1, 2, 4])).sum(1)
    counts = np.bincount(oct_, minlength=8)
    assert counts.min() > 0.7 * 1000 / 8


def test_unreachable_packing_is_an_error():
    import ibemproject_gb300 as g
    L = g.lib()
    num = 400
    C = np.zeros((num, 3))
    R = np.zeros(num)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    p = g.GenParams(num, 0.008, 0.8, 1.2, 0.45, 0.1, g.GEN_RSA, 1, 200000, 0)
    assert L.ibem_e3d_generate_spheres(ctypes.byref(p), dp(C), dp(R), None) == 1
    assert b"stalled" in L.ibem_last_error()
    for bad in (g.GenParams(0, 0.008, 0.8, 1.2, 0.2, 0.1, g.GEN_MC, 1, 0, 0),
                g.GenParams(10, 0.008, 1.2, 0.8, 0.2, 0.1, g.GEN_MC, 1, 0, 0),
                g.GenParams(10, 0.008, 0.8, 1.2, 0.2, 0.1, 7, 1, 0, 0)):
        assert L.ibem_e3d_generate_spheres(ctypes.byref(bad), dp(C), dp(R), None) == 1


def test_matrix_free_helpers_refuse_quadratic_batches():
    """The learned preconditioner, its training data and the autotuner queries take layout 24
    only (the matrix-free solve and products also take layout 60): the Python helpers refuse
    a layout-60 batch before any library call; its row ranges and scalings follow the layout
    (orders 0, 1, 2: a^o / mu0 and a^-o)."""
    import torch

    from ibemproject_gb300 import batch as B
    from ibemproject_gb300 import cases
    cs = [cases.generated_case(n, 0.008, 0.2, seed=n) for n in (3, 5)]
    bt = B.DeviceBatch(cs, device="cpu", layout=60)
    assert bt.N == 60 * 8 and bt.seg_rows(1) == slice(180, 480)
    dr, dc = bt.scalings()
    a = bt.radius_host[0]
    mu0 = cs[0].E0 / (2 * (1 + cs[0].nu0))
    assert np.allclose(dr[:60] * mu0, [1.0] * 6 + [a] * 18 + [a * a] * 36)
    assert np.allclose(dc[:60], [1.0] * 6 + [1 / a] * 18 + [1 / a ** 2] * 36)
    for call in (lambda: B.tuning(bt), lambda: B.tile_shape(bt), lambda: B.training_pairs(bt, 1),
                 lambda: B.training_pairs_mf(bt, 1), lambda: B.prepare(bt)):
        with pytest.raises(ValueError):
            call()


def _pw_max(PA, PB, r):
    """max over lam of the Perram-Wertheim contact function (numpy restatement, grid + refine)."""
    lam = np.linspace(1e-4, 1 - 1e-4, 201)
    best = 0.0
    for _ in range(3):
        vals = [l * (1 - l) * r @ np.linalg.solve((1 - l) * PA + l * PB, r) for l in lam]
        k = int(np.argmax(vals))
        best = max(best, vals[k])
        lo, hi = lam[max(k - 1, 0)], lam[min(k + 1, len(lam) - 1)]
        lam = np.linspace(lo, hi, 41)
    return best


@pytest.mark.parametrize("method,vf", [("rsa", 0.15), ("mc", 0.27)])
def test_ellipsoid_generator_keeps_bodies_apart_and_is_seeded(method, vf):
    """ibem_e3d_generate_ellipsoids: semi-axes in range, unit quaternions, centres in the
    cube, the same microstructure for the same seed, and no two ellipsoids overlapping
    (Perram-Wertheim contact function > 1, checked here by a grid search in numpy); random
    sequential addition and Monte Carlo compression (which reaches the fill fractions where
    addition jams)."""
    from ibemproject_gb300 import cases
    c = cases.ellipsoid_case(150, a1=0.008, vf=vf, seed=2, method=method)
    c2 = cases.ellipsoid_case(150, a1=0.008, vf=vf, seed=2, method=method)
    assert np.array_equal(c.centers, c2.centers) and np.array_equal(c.quats, c2.quats)
    assert not np.array_equal(c.centers, cases.ellipsoid_case(150, a1=0.008, vf=vf, seed=3, method=method).centers)
    A = c.axes
    assert np.all(A[:, 0] == 0.008)
    assert np.all((A[:, 1] >= 0.004) & (A[:, 1] <= 0.008)) and np.all((A[:, 2] >= 0.002) & (A[:, 2] <= 0.008))
    assert np.allclose(np.linalg.norm(c.quats, axis=1), 1.0)
    L = float(c.title.split("=")[1])
    lo = 0.008 if method == "rsa" else 0.0
    assert np.all(c.centers >= lo) and np.all(c.centers <= L - lo)
    vol = (4 / 3 * np.pi * A.prod(axis=1)).sum()
    assert abs(vol / L ** 3 - vf) < 1e-9

    def rot(q):
        w, x, y, z = q / np.linalg.norm(q)
        return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                         [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                         [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    Ps = [rot(q) @ np.diag(a ** 2) @ rot(q).T for q, a in zip(c.quats, A)]
    checked = 0
    for i in range(c.num):
        for j in range(i + 1, c.num):
            r = c.centers[j] - c.centers[i]
            if np.linalg.norm(r) >= A[i, 0] + A[j, 0]:
                continue
            checked += 1
            assert _pw_max(Ps[i], Ps[j], r) > 1.0, (i, j)
    assert checked > 0
