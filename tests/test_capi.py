"""C ABI surface without a GPU: library loads, exports every declared symbol, validates
arguments on the host and computes the ApplyBC plan (a host-only routine)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, case_from_npz, golden

HEADER = os.path.join(ROOT, "include", "ibem_gb300.h")


@pytest.fixture(scope="module")
def g():
    import ibemproject_gb300 as g
    if not os.path.exists(g.LIB_PATH):
        from ibemproject_gb300 import build
        build.build()
    g.lib()
    return g


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_]+\*?\s+\**(ibem_[a-z0-9_]+)\s*\(", txt, re.M)))


def test_header_symbols_exported(g):
    names = declared_symbols()
    assert len(names) >= 14
    for n in names:
        assert hasattr(g.lib(), n), n
        assert n in g.SIGNATURES, n


def test_layout_size(g):
    assert [g.lib().ibem_layout_size(x) for x in (24, 60, 78, 7)] == [24, 60, 78, -1]


def test_argument_errors_without_device(g):
    m = g.material(70e9, 0.3, 400e9, 0.2)
    st = g.lib().ibem_e3d_pair_blocks(None, None, 4, ctypes.byref(m), 25, None, 100, 0, 0, None)
    assert st == g.IBEM_ERR_ARG
    assert b"pair_blocks" in g.lib().ibem_last_error()
    st = g.lib().ibem_e3d_solve(0, -1, None, 0, None, None, 1e-12, None, None)
    assert st == g.IBEM_ERR_ARG


def test_bc_plan_matches_oracle(g, oracle_mod):
    z = golden("example_reference.npz")
    c = case_from_npz(z)
    ucol, tcol = g.bc_plan(c)
    N = 3 * c.NN + 78 * c.num
    H = np.zeros((N, N), order="F")
    G = np.zeros((N, 12 * c.NE), order="F")
    _, _, otcol, t = oracle_mod.apply_bc(c, H, G)
    assert t == 3 * c.NN
    np.testing.assert_array_equal(tcol, otcol)
    flags = c.bc[:, 0]
    assert np.all((ucol >= 0) == (flags == 1))
    assert np.array_equal(ucol[flags == 1], np.arange((flags == 1).sum()))


def test_bc_plan_rejects_non_square(g):
    from ibemproject_gb300 import cases
    c = cases.bounded_cube_case(n_face=2, num=1, grid=0)
    j = int(np.nonzero(c.bc[:, 0] == 1)[0][0])
    c.bc[j, 0] = 0.0   # one more prescribed displacement without a matching traction unknown
    with pytest.raises(g.IbemError):
        g.bc_plan(c)


def test_selftest_bounded_wait_checks_arguments_on_the_host(g):
    assert g.lib().ibem_selftest_bounded_wait(2, 100, None) == g.IBEM_ERR_ARG
    assert g.lib().ibem_selftest_bounded_wait(0, 0, None) == g.IBEM_ERR_ARG
    assert g.lib().ibem_selftest_bounded_wait(1, 1 << 23, None) == g.IBEM_ERR_ARG
