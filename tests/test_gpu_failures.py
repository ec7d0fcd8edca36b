"""Failure paths on the GPU, made without faulting or hanging it.

* Bounded waits: the panel kernel's flag wait and the tensor-core GEMM's mbarrier wait are
  run, through ibem_selftest_bounded_wait, on a flag / barrier that nothing completes, with
  a short poll limit.  Each must give up, raise its error flag and return: the call
  returns IBEM_ERR_TIMEOUT and a normal solve right after it still works.
* Non-convergence: the iterative forms (mixed FP32 LU + GMRES-IR, block-Jacobi GMRES, the
  matrix-free solve) asked for a tolerance below rounding, with their iteration limits,
  return IBEM_ERR_NOCONV, still report the backward error / residual they reached and
  leave the iterate reached in x.
"""
import ctypes

import numpy as np
import pytest

from conftest import scaled_err

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def g():
    import ibemproject_gb300 as g
    g.lib()
    return g


def _small_system(oracle_mod, num=12, seed=3):
    from ibemproject_gb300 import cases
    f = cases.farfield_case(num=num, r0=0.05, vf=0.1, grid=0, seed=seed)
    m = oracle_mod.case_mat(f)
    A = oracle_mod.pair_blocks(f.centers, f.radius, m, 24)
    b = oracle_mod.farfield_rhs(f.num, m, 24, f.sig_inf)
    return f, np.asfortranarray(A), b


def _dense(g, form, A, b, tol, bj_block=0):
    N = len(b)
    At = torch.from_numpy(np.ascontiguousarray(A.T)).cuda()
    bt = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    xt = torch.zeros(N, dtype=torch.float64, device="cuda")
    rep = g.SolveReport()
    P = lambda t: ctypes.c_void_p(t.data_ptr())
    if bj_block:
        st = g.lib().ibem_e3d_solve_bj(N, bj_block, P(At), N, P(bt), P(xt), tol, ctypes.byref(rep), None)
    else:
        st = g.lib().ibem_e3d_solve(form, N, P(At), N, P(bt), P(xt), tol, ctypes.byref(rep), None)
    torch.cuda.synchronize()
    return st, xt.cpu().numpy(), rep


@pytest.mark.parametrize("which", [0, 1])
def test_bounded_wait_gives_up_and_context_stays_usable(g, oracle_mod, which):
    st = g.lib().ibem_selftest_bounded_wait(which, 4096, None)
    assert st == g.IBEM_ERR_TIMEOUT, g.lib().ibem_last_error()
    assert b"gave up" in g.lib().ibem_last_error()
    # the context is intact: a full solve right after it is correct
    _, A, b = _small_system(oracle_mod)
    st, x, rep = _dense(g, g.SOLVE_FP64, A, b, 1e-12)
    assert st == g.IBEM_OK
    assert scaled_err(x, np.linalg.solve(A, b)) < 1e-9


def test_mixed_form_reports_noconv(g, oracle_mod):
    _, A, b = _small_system(oracle_mod)
    st, x, rep = _dense(g, g.SOLVE_MIXED_IR, A, b, 1e-30)
    assert st == g.IBEM_ERR_NOCONV
    assert b"tolerance" in g.lib().ibem_last_error()
    assert 0 < rep.backward_error < 1e-12          # it still got as far as rounding allows
    assert scaled_err(x, np.linalg.solve(A, b)) < 1e-9


def test_block_jacobi_form_reports_noconv(g, oracle_mod):
    _, A, b = _small_system(oracle_mod)
    st, x, rep = _dense(g, g.SOLVE_GMRES_BJ, A, b, 1e-30, bj_block=24)
    assert st == g.IBEM_ERR_NOCONV
    assert 0 < rep.backward_error < 1e-12
    assert scaled_err(x, np.linalg.solve(A, b)) < 1e-9   # the iterate reached is returned


def test_matrix_free_solve_reports_noconv(g):
    from ibemproject_gb300 import batch as B
    from ibemproject_gb300 import cases
    bt = B.DeviceBatch([cases.farfield_case(num=20, r0=0.012, vf=0.15, grid=0, seed=5)])
    b = B.farfield_rhs(bt, np.array([0, 0, 0, 0, 0, 1.0]))
    with pytest.raises(g.IbemError) as ei:
        B.solve(bt, b, B.PRECOND_BLOCK_JACOBI, tol=1e-30, max_outer=1, max_cycles=1)
    assert ei.value.status == g.IBEM_ERR_NOCONV
