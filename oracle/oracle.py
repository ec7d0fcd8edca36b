"""Test infrastructure only: ctypes front end of the oracle (``ibem_oracle.c``).

The oracle is the CPU restatement of the reference's 3D spherical iBEM path used
to check the CUDA library and to time the CPU baseline.  Only the tests, the
smoke check and the bench's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_port", "libibem_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ibem_ref")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_i64 = ctypes.c_int64


class OrcMat(ctypes.Structure):
    _fields_ = [("E0", ctypes.c_double), ("nu0", ctypes.c_double),
                ("E1", ctypes.c_double), ("nu1", ctypes.c_double)]


def build(quiet: bool = True) -> str:
    """Compile the restatement (gcc only; works without the reference sources)."""
    out = subprocess.run(["make", "-C", HERE, "port"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return LIB_PATH


def reference_dir() -> str | None:
    """The reference checkout: IBEM_REFERENCE_DIR, else a directory named ``reference``
    beside the repository; None when neither holds the reference's sources."""
    cands = [os.environ.get("IBEM_REFERENCE_DIR"), os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for d in cands:
        if d and os.path.isfile(os.path.join(d, "integratorElastic3DHelper.cpp")):
            return d
    return None


def build_ref() -> str | None:
    """Compile the reference harness when the reference sources are present."""
    ref = reference_dir()
    if ref is None:
        return None
    out = subprocess.run(["make", "-C", HERE, "ref", f"REF={ref}"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference harness build failed:\n" + out.stdout + out.stderr)
    return REF_BIN


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_layout_size.argtypes = [ctypes.c_int]
        L.orc_D.argtypes = [ctypes.c_int, ctypes.c_int, _dp, ctypes.c_double, ctypes.POINTER(OrcMat), _dp]
        L.orc_IGreen.argtypes = [ctypes.c_int, _dp, ctypes.c_double, ctypes.POINTER(OrcMat), _dp]
        L.orc_Green.argtypes = [ctypes.c_int, _dp, ctypes.POINTER(OrcMat), _dp]
        L.orc_pair_blocks.argtypes = [ctypes.c_int, _dp, _dp, ctypes.POINTER(OrcMat), ctypes.c_int,
                                      _dp, _i64, _i64, _i64]
        L.orc_node_blocks.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, ctypes.POINTER(OrcMat),
                                      ctypes.c_int, _dp, _i64, _i64, _i64]
        L.orc_bem_hg.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, ctypes.POINTER(OrcMat),
                                 _dp, _i64, _i64, _i64, _dp, _i64, _i64, _i64]
        L.orc_bem_to_incl.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _ip, ctypes.c_int, _dp,
                                      ctypes.POINTER(OrcMat), ctypes.c_int, _dp, _i64, _i64, _dp,
                                      _i64, _i64, _i64]
        L.orc_apply_bc.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _dp, _dp, _i64, _dp, _i64, _dp,
                                   _i64, _dp, _i64, _dp, _ip]
        L.orc_get_ut.argtypes = [ctypes.c_int, ctypes.c_int, _i64, _dp, _dp, _ip, _dp, _dp, _dp]
        L.orc_solve_fullpiv.argtypes = [_i64, _dp, _i64, _dp, _dp]
        L.orc_post.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _dp, _dp, ctypes.POINTER(OrcMat),
                               ctypes.c_int, _dp, ctypes.c_int, _dp, ctypes.c_int, _ip, _dp, _dp,
                               _dp, _dp]
        L.orc_stress_kernel.argtypes = [_dp, _dp, ctypes.POINTER(OrcMat), ctypes.c_double,
                                        ctypes.c_double, ctypes.c_int, _dp, _dp]
        L.orc_farfield_rhs.argtypes = [ctypes.c_int, ctypes.POINTER(OrcMat), ctypes.c_int, _dp, _dp]
        L.orc_ell_D_quad.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_double, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, _dp]
        L.orc_ell_I.argtypes = [_ip, _dp, ctypes.c_double, ctypes.c_int]
        L.orc_ell_I.restype = ctypes.c_double
        for f in (L.orc_carlson_rf, L.orc_carlson_rd):
            f.argtypes = [ctypes.c_double] * 3
            f.restype = ctypes.c_double
        L.orc_ell_lambda.argtypes = [_dp, _dp]
        L.orc_ell_lambda.restype = ctypes.c_double
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def mat(E0, nu0, E1, nu1):
    return OrcMat(E0, nu0, E1, nu1)


def case_mat(case):
    """Material record of a case (anything with E0, nu0, E1, nu1)."""
    return OrcMat(case.E0, case.nu0, case.E1, case.nu1)


def layout_size(layout: int) -> int:
    return lib().orc_layout_size(layout)


def D_tensor(order, nder, x, a, m):
    out = np.zeros(3 ** (4 + order + nder))
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib().orc_D(order, nder, _d(x), float(a), ctypes.byref(m), _d(out))
    return out.reshape((3,) * (4 + order + nder))


def IGreen(order, x, a, m):
    out = np.zeros(3 ** (3 + order))
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib().orc_IGreen(order, _d(x), float(a), ctypes.byref(m), _d(out))
    return out.reshape((3,) * (3 + order))


def Green(nder, x, m):
    out = np.zeros(3 ** (2 + nder))
    x = np.ascontiguousarray(x, dtype=np.float64)
    lib().orc_Green(nder, _d(x), ctypes.byref(m), _d(out))
    return out.reshape((3,) * (2 + nder))


def pair_blocks(centers, radius, m, layout):
    centers = np.ascontiguousarray(centers, dtype=np.float64)
    radius = np.ascontiguousarray(radius, dtype=np.float64)
    num = len(radius)
    nu = layout_size(layout)
    n = nu * num
    A = np.zeros((n, n), order="F")
    lib().orc_pair_blocks(num, _d(centers), _d(radius), ctypes.byref(m), layout, _d(A), n, 0, 0)
    return A


def assemble(case, layout, m=None):
    """Full HMAT / GMAT of a bounded case (addBEM, addFieldToBEM, inclusion and
    BEM->inclusion blocks), in the reference's order and layout."""
    m = m or case_mat(case)
    L = lib()
    nu = layout_size(layout)
    NN, NE, num = case.NN, case.NE, case.num
    N = 3 * NN + nu * num
    H = np.zeros((N, N), order="F")
    G = np.zeros((N, 12 * NE), order="F")
    nodes = np.ascontiguousarray(case.nodes, dtype=np.float64)
    conn = np.ascontiguousarray(case.conn, dtype=np.int32)
    cen = np.ascontiguousarray(case.centers, dtype=np.float64)
    rad = np.ascontiguousarray(case.radius, dtype=np.float64)
    if NE:
        L.orc_bem_hg(NN, _d(nodes), NE, _i(conn), ctypes.byref(m), _d(H), N, 0, 0, _d(G), N, 0, 0)
        L.orc_node_blocks(NN, _d(nodes), num, _d(cen), _d(rad), ctypes.byref(m), layout, _d(H), N, 0, 3 * NN)
    L.orc_pair_blocks(num, _d(cen), _d(rad), ctypes.byref(m), layout, _d(H), N, 3 * NN, 3 * NN)
    if NE:
        L.orc_bem_to_incl(NN, _d(nodes), NE, _i(conn), num, _d(cen), ctypes.byref(m), layout,
                          _d(H), N, 0, _d(G), N, 0, 3 * NN)
    return H, G


def apply_bc(case, H, G):
    N = H.shape[0]
    A = np.zeros((N, N), order="F")
    b = np.zeros(N)
    tcol = np.zeros(12 * case.NE, dtype=np.int32)
    conn = np.ascontiguousarray(case.conn, dtype=np.int32)
    bc = np.ascontiguousarray(case.bc, dtype=np.float64)
    tbc = np.ascontiguousarray(case.tbc, dtype=np.float64)
    t = lib().orc_apply_bc(case.NN, case.NE, _i(conn), _d(bc), _d(tbc), N, _d(H), N, _d(G), N,
                           _d(A), N, _d(b), _i(tcol))
    return A, b, tcol, t


def solve_fullpiv(A, b):
    A = np.array(A, order="F", dtype=np.float64, copy=True)
    N = A.shape[0]
    x = np.zeros(N)
    b = np.ascontiguousarray(b, dtype=np.float64)
    rc = lib().orc_solve_fullpiv(N, _d(A), N, _d(b), _d(x))
    if rc != 0:
        raise np.linalg.LinAlgError("singular")
    return x


def get_ut(case, tcol, X):
    N = len(X)
    U = np.zeros(N)
    T = np.zeros(12 * case.NE)
    lib().orc_get_ut(case.NN, case.NE, N, _d(np.ascontiguousarray(case.bc, dtype=np.float64)),
                     _d(np.ascontiguousarray(case.tbc, dtype=np.float64)), _i(tcol),
                     _d(np.ascontiguousarray(X)), _d(U), _d(T))
    return U, T


def post(case, layout, E, Ub=None, Tb=None, sig_inf=None, points=None, m=None):
    m = m or case_mat(case)
    pts = np.ascontiguousarray(case.points if points is None else points, dtype=np.float64)
    nump = len(pts)
    out = np.zeros((nump, 6))
    NE = case.NE
    nodes = np.ascontiguousarray(case.nodes if NE else np.zeros((1, 3)), dtype=np.float64)
    conn = np.ascontiguousarray(case.conn if NE else np.zeros((1, 4)), dtype=np.int32)
    Ub = np.ascontiguousarray(Ub if Ub is not None else np.zeros(1), dtype=np.float64)
    Tb = np.ascontiguousarray(Tb if Tb is not None else np.zeros(1), dtype=np.float64)
    sig = np.ascontiguousarray(sig_inf if sig_inf is not None else np.zeros(6), dtype=np.float64)
    lib().orc_post(nump, _d(pts), case.num, _d(np.ascontiguousarray(case.centers, dtype=np.float64)),
                   _d(np.ascontiguousarray(case.radius, dtype=np.float64)), ctypes.byref(m), layout,
                   _d(np.ascontiguousarray(E, dtype=np.float64)), case.NN, _d(nodes), NE, _i(conn),
                   _d(Ub), _d(Tb), _d(sig), _d(out))
    return out


def farfield_rhs(num, m, layout, sig_inf):
    nu = layout_size(layout)
    b = np.zeros(nu * num)
    lib().orc_farfield_rhs(num, ctypes.byref(m), layout,
                           _d(np.ascontiguousarray(sig_inf, dtype=np.float64)), _d(b))
    return b


def stress_kernel(x, nv, m, dlam, dmu, nder):
    nrow = 6 * 3 ** nder
    Dsu = np.zeros(nrow * 3)
    Dst = np.zeros(nrow * 3)
    lib().orc_stress_kernel(_d(np.ascontiguousarray(x, dtype=np.float64)),
                            _d(np.ascontiguousarray(nv, dtype=np.float64)), ctypes.byref(m),
                            float(dlam), float(dmu), nder, _d(Dsu), _d(Dst))
    return Dsu.reshape(nrow, 3), Dst.reshape(nrow, 3)


# ---------------------------------------------------------------- ellipsoids (ell_oracle.c)
def ell_D_quad(order, nder, x, a, Q, nu, n=(32, 32, 64)):
    """D tensor of an ellipsoid (semi-axes a, rotation Q: Q[i, m] = global component i of
    principal axis m) at the exterior point x (relative to the centre), by volume quadrature
    of the differentiated kernels; digit order as D_tensor."""
    out = np.zeros(3 ** (4 + order + nder))
    lib().orc_ell_D_quad(order, nder, _d(np.ascontiguousarray(x, dtype=np.float64)),
                         _d(np.ascontiguousarray(a, dtype=np.float64)),
                         _d(np.ascontiguousarray(Q, dtype=np.float64).ravel()), float(nu), n[0], n[1], n[2], _d(out))
    return out.reshape((3,) * (4 + order + nder))


def ell_I(k, a, lam, n=64):
    return lib().orc_ell_I(_i(np.ascontiguousarray(k, dtype=np.int32)), _d(np.ascontiguousarray(a, dtype=np.float64)),
                           float(lam), int(n))


def carlson_rf(x, y, z):
    return lib().orc_carlson_rf(x, y, z)


def carlson_rd(x, y, z):
    return lib().orc_carlson_rd(x, y, z)


def ell_lambda(y, a):
    return lib().orc_ell_lambda(_d(np.ascontiguousarray(y, dtype=np.float64)),
                                _d(np.ascontiguousarray(a, dtype=np.float64)))
