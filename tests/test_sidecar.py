"""The binary side-car of a case directory (host/sidecar.cpp; host code, no GPU): the
library reads the same inputs from case.ibemb as from the text files, bit for bit; a text
file newer than the side-car wins; bad side-cars are errors."""
import ctypes
import os
import time

import numpy as np
import pytest


def same(a, b):
    for k in ("E0", "nu0", "E1", "nu1"):
        assert getattr(a, k) == getattr(b, k), k
    for k in ("nodes", "bc", "tbc", "centers", "radius", "points"):
        x, y = np.asarray(getattr(a, k), dtype=np.float64), np.asarray(getattr(b, k), dtype=np.float64)
        assert x.size == y.size and np.array_equal(x.ravel(), y.ravel()), k
    assert np.array_equal(np.asarray(a.conn).ravel(), np.asarray(b.conn).ravel())
    assert (a.sig_inf is None) == (b.sig_inf is None)
    if a.sig_inf is not None:
        assert np.array_equal(a.sig_inf, b.sig_inf)


@pytest.mark.parametrize("kind", ["bounded", "farfield"])
def test_sidecar_reads_what_the_text_files_hold(tmp_path, kind):
    import ibemproject_gb300 as g
    from ibemproject_gb300 import cases
    c = (cases.bounded_cube_case(n_face=3, num=5, radius=0.05, grid=3, seed=3) if kind == "bounded"
         else cases.generated_case(40, 0.01, 0.2, seed=9, grid=4))
    d = str(tmp_path)
    cases.write_case(d, c)
    t, from_sc = g.read_case_native(d)
    assert not from_sc
    same(t, cases.read_case(d))
    same(t, c)
    g.sidecar_from_txt(d)
    s, from_sc = g.read_case_native(d)
    assert from_sc
    same(s, t)
    # a text file edited after the side-car was written wins
    later = time.time() + 5
    os.utime(os.path.join(d, "position.txt"), (later, later))
    _, from_sc = g.read_case_native(d)
    assert not from_sc


def test_sidecar_written_from_arrays_and_bad_files(tmp_path):
    import ibemproject_gb300 as g
    from ibemproject_gb300 import cases
    c = cases.generated_case(25, 0.01, 0.15, seed=4, grid=2)
    d = str(tmp_path)
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (c.centers, c.radius, c.points, c.sig_inf)]
    m = g.material(c.E0, c.nu0, c.E1, c.nu1)
    P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    path = os.path.join(d, "case.ibemb")
    g.check(g.lib().ibem_e3d_sidecar_write(path.encode(), ctypes.byref(m), 0, None, 0, None, None, None, c.num,
                                           P(keep[0]), P(keep[1]), c.nump, P(keep[2]), P(keep[3])))
    s, from_sc = g.read_case_native(d)   # no text files: the side-car is the case
    assert from_sc
    same(s, c)
    raw = open(path, "rb").read()
    open(path, "wb").write(raw[:-8])                  # truncated
    with pytest.raises(g.IbemError):
        g.read_case_native(d)
    open(path, "wb").write(b"NOTACASE" + raw[8:])      # wrong magic
    with pytest.raises(g.IbemError):
        g.read_case_native(d)
