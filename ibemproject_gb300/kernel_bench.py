"""Kernel micro-benchmarks of the dense solver, timed with CUDA events on the launching stream.

  python -m ibemproject_gb300.kernel_bench --gemm 8192,8192,8192 --gemm 24000,24000,8192
  python -m ibemproject_gb300.kernel_bench --lu 16800 --form mixed

--gemm M,N,K   C -= A B in FP32 through ibem_gemm_sub_f32 (split-BF16 x3 tcgen05 kernel).
               Reports the tensor-core kernel alone (algorithmic 2 M N K flops over its
               event time) and the BF16 split kernels.
--lu N         ibem_e3d_solve of a random, diagonally dominant N x N system with the
               per-phase profile (panel, row exchanges, TRSM, GEMM, triangular solves).
--field NUM,G  the double-float stress sums (ibem_e3d_field_form, mixed form) of NUM spheres
               at G^3 grid points with random coefficients: NUM * G^3 pairs per launch.
--solve NUM    the matrix-free solve of one far-field microstructure of NUM spheres (bench
               distribution, N = 24 NUM; --vf sets the volume fraction, 0.15 by default,
               Monte Carlo packing above 0.15) with block-Jacobi, Neumann and learned
               preconditioners (the network trained first on 12 microstructures of 100-150
               spheres): time, Arnoldi and refinement steps, phase times.
--batch R      the batched measurement of bench.py (R realisations of U[50, 500] spheres,
               learned preconditioner, untrained network) with per-phase times.
--quad R       R quadratic-eigenstrain realisations (layout 60, the batched measurement's
               distribution) through ibem_e3d_batch_dense_solve (--quad-form bj: block-Jacobi
               GMRES form, mixed: FP32 LU + GMRES-IR), with phases.
--train-full M the learned preconditioner trained on M microstructures of 500-2,000 spheres
               (pairs from the matrix-free FP64-refined solver, mini-batches), evaluated
               against the small training set, Neumann weights and block-Jacobi.
--post G       ibem_e3d_field (FP64, layout 78) on the bounded-cube case (64 spheres, 600
               boundary elements) at G^3 points: sphere sums and boundary part.
--assemble NUM,LAYOUT  the pair blocks (ibem_e3d_pair_blocks, FP64) of NUM spheres in
               layout 24, 60 or 78: achieved write bandwidth of the N^2 matrix.
--field-far NUM,G  the same with the grid moved far from every sphere (FP32 path only).
--ell NUM,G    ellipsoid pair blocks (FP64) and stress sums (FP64 and mixed) of NUM
               ellipsoids (a1 0.008, a2 a1 U[0.5,1], a3 a1 U[0.25,1], vf 15%) at G^3 points.
--mf NUM       the matrix-free products (ibem_e3d_mf_matvec: FP32, double-float, FP64) on a
               far-field microstructure of NUM spheres (bench distribution): NUM^2 pair
               products per launch, timed by the library's phase events.

One JSON line per case.  The operands are larger than L2 for M, N, K >= 4096; between
repetitions a 256 MB buffer is written to flush L2.
"""
from __future__ import annotations

import argparse
import ctypes
import json

import torch

from . import lib, check, prof_report, SolveReport, SOLVE_FP64, SOLVE_GMRES_BJ, SOLVE_MIXED_IR


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def bench_gemm(m, n, k, reps, dev):
    L = lib()
    g = torch.Generator(device="cpu").manual_seed(7)
    A = torch.randn((k, m), generator=g).to(dev).t()        # column-major m x k
    B = torch.randn((n, k), generator=g).to(dev).t()        # column-major k x n
    C0 = torch.randn((n, m), generator=g).to(dev).t()       # column-major m x n
    C = C0.clone()
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)
    st = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(st.cuda_stream)
    check(L.ibem_gemm_sub_f32(m, n, k, _p(A), m, _p(B), k, _p(C), m, sp))   # warm-up
    torch.cuda.synchronize()
    L.ibem_prof_enable(1)
    for _ in range(reps):
        flush.fill_(1.0)
        check(L.ibem_gemm_sub_f32(m, n, k, _p(A), m, _p(B), k, _p(C), m, sp))
    torch.cuda.synchronize()
    prof = prof_report()
    L.ibem_prof_enable(0)
    tc, sp_ = prof.get("gemm_tc", {}), prof.get("gemm_split", {})
    ms = tc.get("ms", 0.0) / reps
    # accuracy of one product against an FP64 reference on a 256-column slice
    C.copy_(C0)
    check(L.ibem_gemm_sub_f32(m, n, k, _p(A), m, _p(B), k, _p(C), m, sp))
    nc = min(n, 256)
    ref = C0[:, :nc].double() - A.double() @ B[:, :nc].double()
    err = float((C[:, :nc].double() - ref).abs().max() / ref.abs().max())
    return {"kernel": "k_umma_bf16x3", "m": m, "n": n, "k": k, "reps": reps, "ms": ms,
            "tflops_algorithmic": 2.0 * m * n * k / (ms * 1e-3) / 1e12 if ms > 0 else None,
            "tflops_tensor_issued": 6.0 * m * n * k / (ms * 1e-3) / 1e12 if ms > 0 else None,
            "split_ms": sp_.get("ms", 0.0) / reps, "rel_err_vs_fp64": err}


def bench_lu(n, form, reps, dev):
    L = lib()
    g = torch.Generator(device="cpu").manual_seed(11)
    A0 = torch.rand((n, n), generator=g, dtype=torch.float64).to(dev)
    A0 += torch.diag(torch.full((n,), float(n) / 4, dtype=torch.float64, device=dev))
    b = torch.rand(n, generator=g, dtype=torch.float64).to(dev)
    x = torch.empty_like(b)
    st = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(st.cuda_stream)
    rep = SolveReport()
    f = SOLVE_MIXED_IR if form == "mixed" else SOLVE_FP64
    check(L.ibem_e3d_solve(f, n, _p(A0), n, _p(b), _p(x), 1e-12, ctypes.byref(rep), sp))
    torch.cuda.synchronize()
    L.ibem_prof_enable(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        check(L.ibem_e3d_solve(f, n, _p(A0), n, _p(b), _p(x), 1e-12, ctypes.byref(rep), sp))
    e1.record(st)
    torch.cuda.synchronize()
    prof = prof_report()
    L.ibem_prof_enable(0)
    return {"kernel": "dense solve", "n": n, "form": form, "reps": reps, "ms": e0.elapsed_time(e1) / reps,
            "backward_error": rep.backward_error, "iterations": rep.iterations,
            "phases_ms": {k: round(v["ms"] / reps, 3) for k, v in prof.items()},
            "phase_launches": {k: v["launches"] / reps for k, v in prof.items()}}


def bench_assemble(num, layout, reps, dev):
    """ibem_e3d_pair_blocks of a far-field microstructure (bench distribution): the
    (layout num)^2 FP64 matrix written once per call; algorithmic bytes = its 8 N^2 bytes."""
    import numpy as np
    from . import cases, material
    c = cases.farfield_case(num=num, r0=0.012, vf=0.15, grid=0, seed=2024)
    n = layout * num
    A = torch.empty(n * n, dtype=torch.float64, device=dev)
    cen = torch.from_numpy(np.ascontiguousarray(c.centers)).to(dev)
    rad = torch.from_numpy(np.ascontiguousarray(c.radius)).to(dev)
    m = material(c.E0, c.nu0, c.E1, c.nu1)
    st = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(st.cuda_stream)
    L = lib()
    run = lambda: check(L.ibem_e3d_pair_blocks(_p(cen), _p(rad), num, ctypes.byref(m), layout, _p(A), n, 0, 0, sp))
    run()   # warm-up
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        run()
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    return {"kernel": f"pair{layout} + self{layout} (assembly)", "spheres": num, "N": n, "reps": reps, "ms": ms,
            "matrix_GB": 8.0 * n * n / 1e9, "GB_per_s": 8.0 * n * n / (ms * 1e-3) / 1e9,
            "ns_per_pair": ms * 1e6 / (num * num)}


def bench_post(grid, reps, dev):
    """ibem_e3d_field (FP64) on the bounded-cube case of 64 spheres (radius 0.05, 600 Q4
    boundary elements, layout 78) at grid^3 points with random coefficients: the sphere sums
    and the boundary part (phase "bem": quadrature table + Kelvin kernels at 64 Gauss points
    per element and point)."""
    import numpy as np
    from . import cases, material
    c = cases.bounded_cube_case(n_face=10, num=64, radius=0.05, grid=grid, seed=12345)
    rng = np.random.default_rng(5)
    t = lambda a, dt=torch.float64: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dt)
    pts, cen, rad, nodes = t(c.points), t(c.centers), t(c.radius), t(c.nodes)
    conn = t(c.conn, torch.int32)
    E = t(rng.standard_normal(78 * c.num) * 1e-3)
    U = t(rng.standard_normal(3 * c.NN) * 1e-3)
    T = t(rng.standard_normal(12 * c.NE))
    S = torch.empty((c.nump, 6), dtype=torch.float64, device=dev)
    m = material(c.E0, c.nu0, c.E1, c.nu1)
    L = lib()
    run = lambda: check(L.ibem_e3d_field(_p(pts), c.nump, _p(cen), _p(rad), c.num, ctypes.byref(m), 78, _p(E),
                                         _p(nodes), c.NN, _p(conn), c.NE, _p(U), _p(T), None, _p(S), None))
    run()
    torch.cuda.synchronize()
    L.ibem_prof_enable(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        run()
    e1.record()
    torch.cuda.synchronize()
    prof = prof_report()
    L.ibem_prof_enable(0)
    return {"kernel": "field (FP64) with boundary part", "points": c.nump, "elements": c.NE, "spheres": c.num,
            "reps": reps, "ms": e0.elapsed_time(e1) / reps,
            "phases_ms": {k: round(v["ms"] / reps, 3) for k, v in prof.items()},
            "ns_per_point_gauss_point": prof.get("bem", {}).get("ms", 0.0) / reps * 1e6 / (c.nump * c.NE * 64)}


def bench_mf(num, reps, dev):
    from . import batch as B
    from . import cases
    c = cases.farfield_case(num=num, r0=0.012, vf=0.15, grid=0, seed=2024)
    bt = B.DeviceBatch([c], device=dev)
    g = torch.Generator(device="cpu").manual_seed(3)
    x = torch.randn(bt.N, generator=g, dtype=torch.float64).to(dev)
    out = {"kernel": "k_mf_apply", "spheres": num, "pairs": num * num, "reps": reps}
    L = lib()
    for prec, key in ((32, "f32"), (48, "df"), (64, "f64")):
        B.matvec(bt, x, prec)   # warm-up
        L.ibem_prof_enable(1)
        for _ in range(reps):
            B.matvec(bt, x, prec)
        prof = prof_report()
        L.ibem_prof_enable(0)
        ms = prof.get(f"mf_{key}", {}).get("ms", 0.0) / reps
        out[f"{key}_ms"] = ms
        out[f"{key}_ns_per_pair"] = ms * 1e6 / (num * num) if ms > 0 else None
    return out


def bench_field(num, grid, reps, dev, far=False):
    """far: the grid is moved 20 cube sides away, so that every sphere is far from every
    warp's points and only the FP32 path runs (its flop count per pair)."""
    import numpy as np
    from . import Material, batch as B, cases
    c = cases.farfield_case(num=num, r0=0.012, vf=0.15, grid=grid, seed=2024)
    if far:
        c.points = c.points + np.array([20.0 * c.points.max(), 0.0, 0.0])
    L = lib()
    m = Material(c.E0, c.nu0, c.E1, c.nu1)
    g = torch.Generator(device="cpu").manual_seed(5)
    E = (torch.randn(24 * num, generator=g, dtype=torch.float64) * 1e-11).to(dev)
    cen = torch.from_numpy(np.ascontiguousarray(c.centers)).to(dev)
    rad = torch.from_numpy(np.ascontiguousarray(c.radius)).to(dev)
    pts = torch.from_numpy(np.ascontiguousarray(c.points)).to(dev)
    S = torch.empty((c.nump, 6), dtype=torch.float64, device=dev)
    sig = np.ascontiguousarray(c.sig_inf)
    sigp = sig.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    sp = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    run = lambda: check(L.ibem_e3d_field_form(SOLVE_MIXED_IR, _p(pts), c.nump, _p(cen), _p(rad), num, ctypes.byref(m),
                                              24, _p(E), None, 0, None, 0, None, None, sigp, _p(S), sp))
    run()
    torch.cuda.synchronize()
    L.ibem_prof_enable(1)
    for _ in range(reps):
        run()
    prof = prof_report()
    L.ibem_prof_enable(0)
    ms = prof.get("field", {}).get("ms", 0.0) / reps
    pairs = num * c.nump
    return {"kernel": "field24_far + field24_near" + (" (all far: FP32 path)" if far else ""), "spheres": num, "points": c.nump,
            "pairs": pairs, "reps": reps, "ms": ms,
            "ns_per_pair": ms * 1e6 / pairs if ms > 0 else None}


def bench_ell(num, grid, reps, dev):
    """Ellipsoid pair blocks (ibem_e3d_ell_pair_blocks, FP64) and stress sums
    (ibem_e3d_ell_field, FP64 and mixed) of `num` ellipsoids of the config-3 distribution
    (vf 15%) on a grid^3 of points; event-timed per call."""
    import numpy as np
    from . import Material, SOLVE_FP64, SOLVE_MIXED_IR, cases
    c = cases.ellipsoid_case(num, vf=0.15, seed=3, grid=grid)
    L = lib()
    m = Material(c.E0, c.nu0, c.E1, c.nu1)
    N = 24 * num
    dv = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)
    cen, ax, qt, pts = dv(c.centers), dv(c.axes), dv(c.quats), dv(c.points)
    A = torch.empty((N, N), dtype=torch.float64, device=dev)
    E = (torch.randn(N, dtype=torch.float64, generator=torch.Generator().manual_seed(3)) * 1e-9).to(dev)
    S = torch.empty((max(1, c.nump), 6), dtype=torch.float64, device=dev)
    sig = np.ascontiguousarray(c.sig_inf)
    sigp = sig.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    out = {"kernel": "ellipsoids", "num": num, "points": c.nump, "pairs": num * num}

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    out["pair_blocks_ms"] = timed(lambda: check(L.ibem_e3d_ell_pair_blocks(_p(cen), _p(ax), _p(qt), num,
                                                                            ctypes.byref(m), _p(A), N, 0, 0, None)))
    for name, form in (("field_fp64_ms", SOLVE_FP64), ("field_mixed_ms", SOLVE_MIXED_IR)):
        if c.nump:
            out[name] = timed(lambda: check(L.ibem_e3d_ell_field(form, _p(pts), c.nump, _p(cen), _p(ax), _p(qt), num,
                                                                 ctypes.byref(m), _p(E), sigp, _p(S), None)))
    out["ns_per_block"] = out["pair_blocks_ms"] * 1e6 / (num * num)
    if c.nump:
        out["ns_per_field_pair_fp64"] = out["field_fp64_ms"] * 1e6 / (num * c.nump)
    return out


def bench_solve(num, reps, dev, vf=0.15):
    import numpy as np
    from . import batch as B
    from . import cases
    import time
    rng = np.random.default_rng(77)
    train = [cases.farfield_case(num=int(n), r0=0.012, vf=0.15, grid=0, seed=9000 + k)
             for k, n in enumerate(rng.integers(100, 151, size=12))]
    tb = B.DeviceBatch(train, device=dev)
    r, e = B.training_pairs(tb, nrhs=4, seed=5)
    params = B.init_params(seed=1, device=dev)
    hist = B.train(tb, r, e, params, steps=300, lr=3e-3)
    if vf <= 0.15:
        c = cases.farfield_case(num=num, r0=0.012, vf=vf, grid=0, seed=2024)
    else:   # random sequential addition jams near 25%: hard-sphere Monte Carlo packing
        c = cases.generated_case(num, 0.012, vf, seed=2024, method="mc")
    bt = B.DeviceBatch([c], device=dev)
    b = B.farfield_rhs(bt, np.array([0, 0, 0, 0, 0, 1.0]))
    out = {"kernel": "matrix-free solve", "spheres": num, "N": 24 * num, "vf": vf, "reps": reps,
           "training_loss": [float(hist[0]), float(hist[-1])]}
    L = lib()
    for name, pc, pp in (("block_jacobi", B.PRECOND_BLOCK_JACOBI, None), ("neumann", B.PRECOND_NEUMANN, None),
                         ("learned", B.PRECOND_LEARNED, params)):
        B.solve(bt, b, pc, params=pp)   # warm-up
        torch.cuda.synchronize()
        L.ibem_prof_enable(1)
        t = time.perf_counter()
        for _ in range(reps):
            x, rep = B.solve(bt, b, pc, params=pp)
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t) / reps
        prof = prof_report()
        L.ibem_prof_enable(0)
        out[name] = {"s": dt, "arnoldi_steps": rep[0].inner, "refinement_steps": rep[0].outer,
                     "rel_residual": rep[0].rel_residual,
                     "phases_ms": {k: round(v["ms"] / reps, 3) for k, v in prof.items()}}
    return out


def bench_batch(nreal, reps, dev):
    import numpy as np
    from . import batch as B
    from . import cases
    rng = np.random.default_rng(4242)
    nums = rng.integers(50, 501, size=nreal)
    vfs = rng.uniform(0.10, 0.20, size=nreal)
    con = rng.uniform(2.0, 20.0, size=nreal)
    cs = [cases.farfield_case(num=int(n), r0=0.008, vf=float(v), grid=0, seed=7000 + k, E1=70e9 * float(c))
          for k, (n, v, c) in enumerate(zip(nums, vfs, con))]
    bt = B.DeviceBatch(cs, device=dev)
    params = B.init_params(seed=1, device=dev)
    b = B.farfield_rhs(bt, np.array([0, 0, 0, 0, 0, 1.0]))
    B.solve(bt, b, B.PRECOND_LEARNED, params=params)   # warm-up (and tuning)
    L = lib()
    L.ibem_prof_enable(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        x, rep = B.solve(bt, b, B.PRECOND_LEARNED, params=params)
    e1.record()
    torch.cuda.synchronize()
    prof = prof_report()
    L.ibem_prof_enable(0)
    return {"kernel": "batched matrix-free solve", "realisations": nreal, "spheres": int(nums.sum()),
            "ms": e0.elapsed_time(e1) / reps, "arnoldi_steps_max": max(r.inner for r in rep),
            "phases_ms": {k: round(v["ms"] / reps, 3) for k, v in prof.items()},
            "phase_launches": {k: v["launches"] / reps for k, v in prof.items()}}


def bench_quad(nreal, reps, dev, form="bj"):
    """Quadratic-eigenstrain realisations of the batched measurement's distribution (U[50,
    500] spheres, vf U[10%, 30%], E1/E0 U[2, 20], layout 60) through
    ibem_e3d_batch_dense_solve (mixed form), with the per-phase profile."""
    import numpy as np
    from . import batch as B
    from . import cases
    rng = np.random.default_rng(4243)
    nums = rng.integers(50, 501, size=nreal)
    vfs = rng.uniform(0.10, 0.30, size=nreal)
    con = rng.uniform(2.0, 20.0, size=nreal)
    cs = [cases.generated_case(int(n), 0.008, float(v), seed=7500 + k, E1=70e9 * float(c))
          for k, (n, v, c) in enumerate(zip(nums, vfs, con))]
    bt = B.DeviceBatch(cs, device=dev, layout=60)
    b = B.farfield_rhs(bt, np.array([0, 0, 0, 0, 0, 1.0]))
    f = SOLVE_GMRES_BJ if form == "bj" else SOLVE_MIXED_IR
    B.dense_batch_solve(bt, b, f, tol=1e-12)   # warm-up
    torch.cuda.synchronize()
    L = lib()
    L.ibem_prof_enable(1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        x, rep = B.dense_batch_solve(bt, b, f, tol=1e-12)
    e1.record()
    torch.cuda.synchronize()
    prof = prof_report()
    L.ibem_prof_enable(0)
    return {"kernel": "batched dense solves, layout 60", "form": form, "realisations": nreal, "spheres": int(nums.sum()),
            "unknowns": int(60 * nums.sum()), "ms": e0.elapsed_time(e1) / reps,
            "factor_ms_sum": sum(r.t_factor_ms for r in rep), "solve_ms_sum": sum(r.t_solve_ms for r in rep),
            "gmres_iterations_max": max(r.iterations for r in rep),
            "phases_ms": {k: round(v["ms"] / reps, 3) for k, v in prof.items()},
            "phase_launches": {k: v["launches"] / reps for k, v in prof.items()}}


def _eval_preconditioners(c, variants, dev, reps=2):
    """Matrix-free solve of one far-field microstructure with each (name, precond, params)."""
    import time
    import numpy as np
    from . import batch as B
    bt = B.DeviceBatch([c], device=dev)
    b = B.farfield_rhs(bt, np.array([0, 0, 0, 0, 0, 1.0]))
    out = {}
    for name, pc, pp in variants:
        B.solve(bt, b, pc, params=pp)
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            _, rep = B.solve(bt, b, pc, params=pp)
        torch.cuda.synchronize()
        out[name] = {"s": (time.perf_counter() - t) / reps, "arnoldi_steps": rep[0].inner,
                     "refinement_steps": rep[0].outer, "rel_residual": rep[0].rel_residual}
    return out


def bench_train_full(nmicro, steps, dev, groups=10, nrhs=2):
    """The learned preconditioner trained on the full-size training set: nmicro seeded
    microstructures of U[500, 2000] spheres (radius U[0.8, 1.2] x 0.012, Monte Carlo packing,
    vf U[15%, 25%], E1/E0 U[2, 20]), nrhs residual / correction pairs each from the
    matrix-free FP64-refined solver (relative residual 1e-10), mini-batches of nmicro / groups
    microstructures cycled over `steps` AdamW steps; against the small set (12
    microstructures of 100-150 spheres, dense FP64 pairs, full batch), the analytic Neumann
    weights and block-Jacobi, on the 2,000-sphere bench microstructure and on 20,000 spheres
    at vf 25%."""
    import time
    import numpy as np
    from . import batch as B
    from . import cases
    rng = np.random.default_rng(31)
    nums = rng.integers(500, 2001, size=nmicro)
    vfs = rng.uniform(0.15, 0.25, size=nmicro)
    con = rng.uniform(2.0, 20.0, size=nmicro)
    t = time.perf_counter()
    cs = [cases.generated_case(int(n), 0.012, float(v), seed=20000 + k, E1=70e9 * float(c0))
          for k, (n, v, c0) in enumerate(zip(nums, vfs, con))]
    t_gen = time.perf_counter() - t
    t = time.perf_counter()
    preps = []
    per = (nmicro + groups - 1) // groups
    for g0 in range(0, nmicro, per):
        bt = B.DeviceBatch(cs[g0:g0 + per], device=dev)
        r, e = B.training_pairs_mf(bt, nrhs, seed=g0)
        preps.append((B.prepare(bt, r, e), bt.num))
        del r, e
    torch.cuda.synchronize()
    t_pairs = time.perf_counter() - t
    params = B.init_params(seed=1, device=dev)
    m = torch.zeros_like(params)
    v = torch.zeros_like(params)
    first = [B.loss_grad(p, n, params)[0] for p, n in preps]
    t = time.perf_counter()
    for it in range(steps):
        p, n = preps[it % len(preps)]
        _, gr = B.loss_grad(p, n, params)
        B.adamw(params, gr, m, v, it + 1, 3e-3)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t
    last = [B.loss_grad(p, n, params)[0] for p, n in preps]
    del preps
    # the small training set of bench.py
    rs = np.random.default_rng(77)
    sn = rs.integers(100, 151, size=12)
    sv = rs.uniform(0.10, 0.20, size=12)
    sc = rs.uniform(2.0, 20.0, size=12)
    sc[:4] = 400.0 / 70.0
    small = [cases.farfield_case(num=int(n), r0=0.012, vf=float(v0), grid=0, seed=9000 + k, E1=70e9 * float(c0))
             for k, (n, v0, c0) in enumerate(zip(sn, sv, sc))]
    sb = B.DeviceBatch(small, device=dev)
    r, e = B.training_pairs(sb, nrhs=4, seed=5)
    ps = B.init_params(seed=1, device=dev)
    B.train(sb, r, e, ps, steps=300, lr=3e-3)
    variants = [("block_jacobi", B.PRECOND_BLOCK_JACOBI, None), ("neumann", B.PRECOND_NEUMANN, None),
                ("learned_small_set", B.PRECOND_LEARNED, ps), ("learned_full_set", B.PRECOND_LEARNED, params)]
    ev = {"bench_2000_vf15": _eval_preconditioners(cases.farfield_case(num=2000, r0=0.012, vf=0.15, grid=0, seed=2024),
                                                   variants, dev),
          "spheres_20000_vf25": _eval_preconditioners(cases.generated_case(20000, 0.012, 0.25, seed=2024), variants,
                                                      dev, reps=1)}
    return {"kernel": "learned preconditioner, full training set", "microstructures": nmicro,
            "spheres": int(nums.sum()), "pairs": nrhs * nmicro, "groups": len(first), "steps": steps,
            "generation_s": t_gen, "pairs_and_graphs_s": t_pairs, "train_s": t_train,
            "loss_first_mean": float(np.mean(first)), "loss_last_mean": float(np.mean(last)), "evaluation": ev}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gemm", action="append", default=[], help="M,N,K")
    ap.add_argument("--lu", type=int, action="append", default=[])
    ap.add_argument("--form", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--mf", type=int, action="append", default=[])
    ap.add_argument("--field", action="append", default=[], help="NUM,GRID")
    ap.add_argument("--field-far", action="append", default=[], help="NUM,GRID with every sphere far from the points")
    ap.add_argument("--ell", action="append", default=[], help="NUM,GRID: ellipsoid pair blocks and stress sums")
    ap.add_argument("--solve", type=int, action="append", default=[])
    ap.add_argument("--batch", type=int, action="append", default=[])
    ap.add_argument("--assemble", action="append", default=[], help="NUM,LAYOUT")
    ap.add_argument("--quad", type=int, action="append", default=[])
    ap.add_argument("--train-full", type=int, default=0, help="microstructures of the full training set")
    ap.add_argument("--train-steps", type=int, default=300)
    ap.add_argument("--post", type=int, action="append", default=[], help="grid of the bounded-cube field")
    ap.add_argument("--quad-form", default="bj", choices=["bj", "mixed"])
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--vf", type=float, default=0.15, help="volume fraction of --solve (above 0.15: Monte Carlo packing)")
    a = ap.parse_args(argv)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    for s in a.gemm:
        m, n, k = (int(v) for v in s.split(","))
        print(json.dumps(bench_gemm(m, n, k, a.reps, dev)), flush=True)
    for n in a.lu:
        print(json.dumps(bench_lu(n, a.form, a.reps, dev)), flush=True)
    for f in a.assemble:
        num, lay = (int(v) for v in f.split(","))
        print(json.dumps(bench_assemble(num, lay, a.reps, dev)), flush=True)
    for n in a.mf:
        print(json.dumps(bench_mf(n, a.reps, dev)), flush=True)
    if a.train_full:
        print(json.dumps(bench_train_full(a.train_full, a.train_steps, dev)), flush=True)
    for gsz in a.post:
        print(json.dumps(bench_post(gsz, a.reps, dev)), flush=True)
    for n in a.quad:
        print(json.dumps(bench_quad(n, a.reps, dev, a.quad_form)), flush=True)
    for n in a.solve:
        print(json.dumps(bench_solve(n, a.reps, dev, a.vf)), flush=True)
    for n in a.batch:
        print(json.dumps(bench_batch(n, a.reps, dev)), flush=True)
    for f in a.field:
        num, grid = (int(v) for v in f.split(","))
        print(json.dumps(bench_field(num, grid, a.reps, dev)), flush=True)
    for f in a.ell:
        num, grid = (int(v) for v in f.split(","))
        print(json.dumps(bench_ell(num, grid, a.reps, dev)), flush=True)
    for f in a.field_far:
        num, grid = (int(v) for v in f.split(","))
        print(json.dumps(bench_field(num, grid, a.reps, dev, far=True)), flush=True)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
