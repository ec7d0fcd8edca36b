"""Kernel-level parity of the CUDA path (through the C ABI) with the oracle and with the
reference's own matrices.  Tolerance: 1e-11 of the largest entry of the compared block
for matrix entries (all FP64)."""
import ctypes

import numpy as np
import pytest

from conftest import case_from_npz, golden, scaled_err

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

MAT = (70e9, 0.3, 400e9, 0.2)


def dev(a, dtype=None):
    a = np.ascontiguousarray(a)
    t = torch.from_numpy(a)
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def P(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.fixture(scope="module")
def g():
    import ibemproject_gb300 as g
    assert torch.cuda.is_available(), "GPU tests need CUDA"
    g.lib()
    return g


def spheres(n, seed):
    from ibemproject_gb300 import cases
    rng = np.random.default_rng(seed)
    C, R = cases.rsa_spheres(n, rng, 0.15, 0.85, lambda k: 0.03 + 0.03 * ((k * 7) % 5) / 5,
                             lambda r, Rk: r + Rk + 0.01)
    return C, R


@pytest.mark.parametrize("layout", [24, 60, 78])
def test_pair_blocks_vs_oracle(g, oracle_mod, layout):
    C, R = spheres(6, 3)
    m = g.material(*MAT)
    want = oracle_mod.pair_blocks(C, R, oracle_mod.mat(*MAT), layout)
    n = layout * len(R)
    pad = 5
    # torch is row-major: a (cols x rows) tensor is the column-major (rows x cols) matrix
    At = torch.full((n + 3 * pad, n + 2 * pad), float("nan"), dtype=torch.float64, device="cuda")
    dC, dR = dev(C), dev(R)   # keep the device copies alive until the kernel has run
    g.check(g.lib().ibem_e3d_pair_blocks(P(dC), P(dR), len(R), ctypes.byref(m), layout, P(At),
                                         At.shape[1], pad, 2 * pad, None))
    torch.cuda.synchronize()
    got = At.cpu().numpy().T   # column-major view: got[r, c] = At[c, r]
    blk = got[pad:pad + n, 2 * pad:2 * pad + n]
    for s in range(len(R)):
        for h in range(len(R)):
            sl = (slice(layout * s, layout * (s + 1)), slice(layout * h, layout * (h + 1)))
            assert scaled_err(blk[sl], want[sl]) < 1e-11
    # nothing written outside the block
    mask = np.ones_like(got, dtype=bool)
    mask[pad:pad + n, 2 * pad:2 * pad + n] = False
    assert np.all(np.isnan(got[mask]))


@pytest.mark.parametrize("layout", [24, 78])
def test_node_blocks_vs_oracle(g, oracle_mod, layout):
    from ibemproject_gb300 import cases
    nodes, conn, face = cases.cube_mesh(3)
    C, R = spheres(3, 5)
    m = g.material(*MAT)
    NN = len(nodes)
    H = torch.zeros((layout * len(R), 3 * NN), dtype=torch.float64, device="cuda")  # column-major 3NN x nu*num
    dn, dC, dR = dev(nodes), dev(C), dev(R)
    g.check(g.lib().ibem_e3d_node_blocks(P(dn), NN, P(dC), P(dR), len(R), ctypes.byref(m), layout,
                                         P(H), 3 * NN, 0, 0, None))
    torch.cuda.synchronize()
    got = H.cpu().numpy().T
    want = np.zeros((3 * NN, layout * len(R)), order="F")
    _d = ctypes.POINTER(ctypes.c_double)
    oracle_mod.lib().orc_node_blocks(NN, nodes.ctypes.data_as(_d), len(R), np.ascontiguousarray(C).ctypes.data_as(_d),
                                     np.ascontiguousarray(R).ctypes.data_as(_d), ctypes.byref(oracle_mod.mat(*MAT)),
                                     layout, want.ctypes.data_as(_d), 3 * NN, 0, 0)
    assert scaled_err(got, want) < 1e-11


def _tiny_device_matrices(g, layout=78):
    z = golden("tiny_reference.npz")
    c = case_from_npz(z)
    m = g.material(c.E0, c.nu0, c.E1, c.nu1)
    N = 3 * c.NN + layout * c.num
    Ht = torch.zeros((N, N), dtype=torch.float64, device="cuda")
    Gt = torch.zeros((12 * c.NE, N), dtype=torch.float64, device="cuda")
    nodes, conn, cen, rad = dev(c.nodes), dev(c.conn.astype(np.int32)), dev(c.centers), dev(c.radius)
    L = g.lib()
    g.check(L.ibem_e3d_bem_hg(P(nodes), c.NN, P(conn), c.NE, ctypes.byref(m), P(Ht), N, 0, 0, P(Gt), N, 0, 0, None))
    g.check(L.ibem_e3d_node_blocks(P(nodes), c.NN, P(cen), P(rad), c.num, ctypes.byref(m), layout, P(Ht), N, 0,
                                   3 * c.NN, None))
    g.check(L.ibem_e3d_pair_blocks(P(cen), P(rad), c.num, ctypes.byref(m), layout, P(Ht), N, 3 * c.NN, 3 * c.NN,
                                   None))
    g.check(L.ibem_e3d_bem_to_incl(P(nodes), c.NN, P(conn), c.NE, P(cen), c.num, ctypes.byref(m), layout, P(Ht), N,
                                   0, P(Gt), N, 0, 3 * c.NN, None))
    torch.cuda.synchronize()
    del nodes, conn, cen, rad
    return z, c, Ht, Gt


def test_assembly_vs_reference_matrices(g):
    z, c, Ht, Gt = _tiny_device_matrices(g)
    H = Ht.cpu().numpy().T
    G = Gt.cpu().numpy().T
    n3 = 3 * c.NN
    for rs, cs in [(slice(0, n3), slice(0, n3)), (slice(0, n3), slice(n3, None)),
                   (slice(n3, None), slice(n3, None)), (slice(n3, None), slice(0, n3))]:
        assert scaled_err(H[rs, cs], z["HMAT"][rs, cs]) < 1e-11
    assert scaled_err(G[:n3], z["GMAT"][:n3]) < 1e-11
    assert scaled_err(G[n3:], z["GMAT"][n3:]) < 1e-11


def test_assembly_is_bit_reproducible(g):
    """H sums element contributions per node in a fixed order (no atomics on matrix
    entries): two assemblies of a mesh whose nodes are shared by up to four elements give
    the same matrices bit for bit."""
    from ibemproject_gb300 import cases
    c = cases.bounded_cube_case(n_face=4, num=3, radius=0.1, grid=0, seed=11)
    mats = []
    for _ in range(2):
        m = g.material(c.E0, c.nu0, c.E1, c.nu1)
        N = 3 * c.NN + 24 * c.num
        Ht = torch.zeros((N, N), dtype=torch.float64, device="cuda")
        Gt = torch.zeros((12 * c.NE, N), dtype=torch.float64, device="cuda")
        nodes, conn, cen = dev(c.nodes), dev(c.conn.astype(np.int32)), dev(c.centers)
        L = g.lib()
        g.check(L.ibem_e3d_bem_hg(P(nodes), c.NN, P(conn), c.NE, ctypes.byref(m), P(Ht), N, 0, 0, P(Gt), N, 0, 0,
                                  None))
        g.check(L.ibem_e3d_bem_to_incl(P(nodes), c.NN, P(conn), c.NE, P(cen), c.num, ctypes.byref(m), 24, P(Ht),
                                       N, 0, P(Gt), N, 0, 3 * c.NN, None))
        torch.cuda.synchronize()
        mats.append((Ht.cpu(), Gt.cpu()))
    assert torch.equal(mats[0][0], mats[1][0]) and torch.equal(mats[0][1], mats[1][1])
    assert mats[0][0].abs().max() > 0


def test_apply_bc_and_get_ut(g, oracle_mod):
    z, c, Ht, Gt = _tiny_device_matrices(g)
    N = Ht.shape[0]
    ucol, tcol = g.bc_plan(c)
    At = torch.zeros((N, N), dtype=torch.float64, device="cuda")
    b = torch.zeros(N, dtype=torch.float64, device="cuda")
    bc, tbc = dev(c.bc), dev(c.tbc)
    du, dt = dev(ucol), dev(tcol)
    g.check(g.lib().ibem_e3d_apply_bc(c.NN, c.NE, N, P(du), P(dt), P(bc), P(tbc), P(Ht), N, P(Gt), N, P(At), N,
                                      P(b), None))
    torch.cuda.synchronize()
    A_o, b_o, _, _ = oracle_mod.apply_bc(c, z["HMAT"], z["GMAT"])
    assert scaled_err(At.cpu().numpy().T, A_o) < 1e-11
    assert scaled_err(b.cpu().numpy(), z["b"]) < 1e-11
    X = dev(z["X"])
    U = torch.zeros(N, dtype=torch.float64, device="cuda")
    T = torch.zeros(12 * c.NE, dtype=torch.float64, device="cuda")
    g.check(g.lib().ibem_e3d_get_ut(c.NN, c.NE, N, P(du), P(dt), P(bc), P(tbc), P(X), P(U), P(T), None))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(U.cpu().numpy(), z["U"])
    np.testing.assert_array_equal(T.cpu().numpy(), z["T"])


@pytest.mark.parametrize("form", [0, 1])
def test_solve_tiny_reference_system(g, oracle_mod, form):
    z = golden("tiny_reference.npz")
    c = case_from_npz(z)
    A_o, b_o, _, _ = oracle_mod.apply_bc(c, z["HMAT"], z["GMAT"])
    N = len(b_o)
    At = dev(np.asfortranarray(A_o).T.copy())  # row-major torch holding A^T == column-major A
    b = dev(b_o)
    x = torch.zeros(N, dtype=torch.float64, device="cuda")
    rep = g.SolveReport()
    g.check(g.lib().ibem_e3d_solve(form, N, P(At), N, P(b), P(x), 1e-13, ctypes.byref(rep), None))
    xs = x.cpu().numpy()
    n3 = 3 * c.NN
    assert scaled_err(xs[n3:], z["X"][n3:]) < 1e-9
    assert scaled_err(xs[:n3], z["X"][:n3]) < 1e-9
    assert rep.backward_error < 1e-13


def test_field_vs_oracle(g, oracle_mod):
    z = golden("tiny_reference.npz")
    c = case_from_npz(z)
    m = g.material(c.E0, c.nu0, c.E1, c.nu1)
    n3 = 3 * c.NN
    E = z["U"][n3:]
    S = torch.zeros((c.nump, 6), dtype=torch.float64, device="cuda")
    keep = [dev(c.points), dev(c.centers), dev(c.radius), dev(E), dev(c.nodes), dev(c.conn.astype(np.int32)),
            dev(z["U"]), dev(z["T"])]
    pts, cen, rad, dE, nodes, conn, dU, dT = keep
    g.check(g.lib().ibem_e3d_field(P(pts), c.nump, P(cen), P(rad), c.num, ctypes.byref(m), 78, P(dE), P(nodes),
                                   c.NN, P(conn), c.NE, P(dU), P(dT), None, P(S), None))
    torch.cuda.synchronize()
    assert scaled_err(S.cpu().numpy(), z["stress"]) < 1e-11


@pytest.mark.parametrize("m,n,k", [(256, 256, 64), (300, 520, 200), (1024, 768, 1000), (129, 257, 33)])
def test_tensor_core_gemm(g, m, n, k):
    """C -= A B on the tcgen05 tensor cores with split-BF16 operands: close to FP32 (the
    dropped lo*lo term is ~2^-16 relative per product; tolerance 2e-5 of max|A||B| k)."""
    gen = torch.Generator(device="cpu").manual_seed(m + n + k)
    A = torch.randn(k, m, generator=gen, dtype=torch.float32).cuda()   # column-major m x k (lda = m)
    B = torch.randn(n, k, generator=gen, dtype=torch.float32).cuda()   # column-major k x n (ldb = k)
    C = torch.randn(n, m, generator=gen, dtype=torch.float32).cuda()   # column-major m x n (ldc = m)
    want = C.double() - (A.double().T @ B.double().T).T
    g.check(g.lib().ibem_gemm_sub_f32(m, n, k, P(A), m, P(B), k, P(C), m, None))
    torch.cuda.synchronize()
    err = (C.double() - want).abs().max().item()
    scale = (A.abs().max() * B.abs().max()).item() * k
    assert err < 2e-5 * scale, (err, scale)
    # and much better than a plain BF16 product would be
    assert err < 1e-4 * (A.double().T @ B.double().T).abs().max().item()


@pytest.mark.gpu
def test_field_double_float_vs_fp64_and_oracle(g, oracle_mod):
    """Stresses of the 24-unknown layout: the FP64 sums match the oracle to 1e-11 and the
    split sums of the mixed form (ibem_e3d_field_form: double-float for spheres within 12
    radii of a warp's points, FP32 beyond) to 1e-9 (scaled), with points inside, near and
    far from the spheres.  The FP32 share is designed for ~1e-9 of the strain (random-sign
    coefficients, as here, are its worst case); the solution target is 1e-8."""
    from ibemproject_gb300 import cases
    c = cases.farfield_case(num=60, r0=0.05, vf=0.15, grid=10, seed=3)
    rng = np.random.default_rng(4)
    E = rng.normal(size=(c.num, 24)) * 1e-3
    E[:, 6:] /= 0.05   # order-1 eigenstrain per unit length
    E = E.ravel()
    m = g.material(c.E0, c.nu0, c.E1, c.nu1)
    sig = np.ascontiguousarray(c.sig_inf, dtype=np.float64)
    sigp = sig.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    keep = [dev(c.points), dev(c.centers), dev(c.radius), dev(E)]
    pts, cen, rad, dE = keep
    out = {}
    for form in (g.SOLVE_FP64, g.SOLVE_MIXED_IR):
        S = torch.zeros((c.nump, 6), dtype=torch.float64, device="cuda")
        g.check(g.lib().ibem_e3d_field_form(form, P(pts), c.nump, P(cen), P(rad), c.num, ctypes.byref(m), 24, P(dE),
                                            None, 0, None, 0, None, None, sigp, P(S), None))
        torch.cuda.synchronize()
        out[form] = S.cpu().numpy()
    ref = oracle_mod.post(c, 24, E, sig_inf=c.sig_inf)
    assert scaled_err(out[g.SOLVE_FP64], ref) < 1e-11
    assert scaled_err(out[g.SOLVE_MIXED_IR], ref) < 1e-9
    assert scaled_err(out[g.SOLVE_MIXED_IR], out[g.SOLVE_FP64]) < 1e-9
