"""Input data of the 3D spherical iBEM path: the reference's txt formats and
seeded synthetic microstructures.

Formats (read exactly as the reference reads them):

* ``position.txt`` -- ``num E1 nu1`` then ``num`` rows ``x y z a``
  (configElastic3D.cpp:106-128, whitespace-separated ``>>`` reads).
* ``BEM.txt`` -- five header lines (title, E0, nu0, NN, NE; read with ``getline``,
  configElastic3D.cpp:32-71), then whitespace-separated NN x 3 node coordinates,
  NE x 4 one-based Q4 connectivity, 3NN x 2 displacement conditions
  (flag 1 = unknown, 0 = prescribed; value) and NE x 24 traction conditions
  (12 flags, 12 values) (configElastic3D.cpp:73-93).
* ``postprocess.txt`` -- ``nump`` then ``nump`` rows ``x y z`` (configElastic3D.h:116-129).

The reference files use CR-only and CR-CR-LF line ends; both are accepted.
A case with NN = NE = 0 has no boundary and is loaded by a far-field stress
``sig_inf`` (xx xy xz yy yz zz) instead; the reference has no such loading, so
such cases are written with an empty ``BEM.txt`` body plus ``farfield.txt``.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np


@dataclasses.dataclass
class Case:
    E0: float
    nu0: float
    E1: float
    nu1: float
    nodes: np.ndarray          # NN x 3
    conn: np.ndarray           # NE x 4, one-based, int32
    bc: np.ndarray             # 3NN x 2
    tbc: np.ndarray            # NE x 24
    centers: np.ndarray        # num x 3
    radius: np.ndarray         # num
    points: np.ndarray         # nump x 3
    sig_inf: np.ndarray | None = None   # far-field stress (6) for boundary-free cases
    title: str = "ibem_case"
    axes: np.ndarray | None = None      # ellipsoids: num x 3 semi-axes (None: spheres of `radius`)
    quats: np.ndarray | None = None     # ellipsoids: num x 4 unit quaternions (w, x, y, z)

    @property
    def NN(self) -> int:
        return int(self.nodes.shape[0])

    @property
    def NE(self) -> int:
        return int(self.conn.shape[0])

    @property
    def num(self) -> int:
        return int(self.radius.shape[0])

    @property
    def nump(self) -> int:
        return int(self.points.shape[0])

    def n_unknowns(self, layout: int) -> int:
        return 3 * self.NN + layout * self.num


def _lines(path: str) -> list[str]:
    with open(path, "rb") as f:
        txt = f.read().decode("latin-1")
    return txt.split("\n")


def read_case(path: str) -> Case:
    """Load the three reference input files (plus ``farfield.txt`` when present)."""
    with open(os.path.join(path, "position.txt"), "rb") as f:
        tok = f.read().decode("latin-1").split()
    num = int(tok[0])
    E1, nu1 = float(tok[1]), float(tok[2])
    pv = np.array(tok[3:3 + 4 * num], dtype=np.float64).reshape(num, 4)

    lines = _lines(os.path.join(path, "BEM.txt"))
    head = [ln.strip("\r") for ln in lines[:5]]
    title = head[0]
    E0, nu0 = float(head[1]), float(head[2])
    NN, NE = int(head[3]), int(head[4])
    body = " ".join(lines[5:]).split()
    o = 0
    nodes = np.array(body[o:o + 3 * NN], dtype=np.float64).reshape(NN, 3); o += 3 * NN
    conn = np.array(body[o:o + 4 * NE], dtype=np.float64).astype(np.int32).reshape(NE, 4); o += 4 * NE
    bc = np.array(body[o:o + 6 * NN], dtype=np.float64).reshape(3 * NN, 2); o += 6 * NN
    tbc = np.array(body[o:o + 24 * NE], dtype=np.float64).reshape(NE, 24); o += 24 * NE

    with open(os.path.join(path, "postprocess.txt"), "rb") as f:
        tok = f.read().decode("latin-1").split()
    nump = int(tok[0])
    pts = np.array(tok[1:1 + 3 * nump], dtype=np.float64).reshape(nump, 3)

    sig = None
    ff = os.path.join(path, "farfield.txt")
    if os.path.exists(ff):
        with open(ff) as f:
            sig = np.array(f.read().split()[:6], dtype=np.float64)
    return Case(E0, nu0, E1, nu1, nodes, conn, bc, tbc, pv[:, :3].copy(), pv[:, 3].copy(), pts,
                sig, title)


def _f(v) -> str:
    """Shortest round-trip decimal of a float (read back bit-exactly by strtod / >>)."""
    return repr(float(v))


def write_case(path: str, c: Case) -> None:
    os.makedirs(path, exist_ok=True)
    with open(os.path.join(path, "position.txt"), "w") as f:
        f.write(f"{c.num}\n{_f(c.E1)}\n{_f(c.nu1)}\n")
        for p, a in zip(c.centers, c.radius):
            f.write(f"{_f(p[0])} {_f(p[1])} {_f(p[2])} {_f(a)}\n")
    with open(os.path.join(path, "BEM.txt"), "w") as f:
        f.write(f"{c.title}\n{_f(c.E0)}\n{_f(c.nu0)}\n{c.NN}\n{c.NE}\n\n")
        for p in c.nodes:
            f.write(f"{_f(p[0])} {_f(p[1])} {_f(p[2])}\n")
        for e in c.conn:
            f.write(" ".join(str(int(v)) for v in e) + "\n")
        for r in c.bc:
            f.write(f"{int(r[0])} {_f(r[1])}\n")
        for r in c.tbc:
            f.write(" ".join(str(int(v)) for v in r[:12]) + " " + " ".join(_f(v) for v in r[12:]) + "\n")
    with open(os.path.join(path, "postprocess.txt"), "w") as f:
        f.write(f"{c.nump}\n")
        for p in c.points:
            f.write(f"{_f(p[0])} {_f(p[1])} {_f(p[2])}\n")
    ff = os.path.join(path, "farfield.txt")
    if c.sig_inf is not None:
        with open(ff, "w") as f:
            f.write(" ".join(_f(v) for v in c.sig_inf) + "\n")
    elif os.path.exists(ff):
        os.remove(ff)


# --------------------------------------------------------------------------
# Synthetic inputs

def cube_mesh(n: int, side: float = 1.0):
    """Surface of the cube [0, side]^3 meshed by n x n Q4 elements per face.

    Returns (nodes NN x 3, conn NE x 4 one-based, face id per element).  Corner
    order gives the outward normal through (x2 - x1) x (x4 - x1), the convention
    of Normal_Jac (BEMElasticHelper3D.cpp:226-267).  NN = 6 n^2 + 2, NE = 6 n^2.
    """
    g = np.linspace(0.0, side, n + 1)
    key_of = {}
    nodes = []

    def nid(p):
        k = tuple(int(round(v / side * n)) for v in p)
        if k not in key_of:
            key_of[k] = len(nodes)
            nodes.append(p)
        return key_of[k] + 1

    conn, face = [], []
    # (origin, u, v) chosen so that u x v points outward
    L = side
    faces = [
        (np.array([0, 0, 0.0]), np.array([0, 1, 0.0]), np.array([1, 0, 0.0])),   # z = 0, normal -z
        (np.array([0, 0, L]), np.array([1, 0, 0.0]), np.array([0, 1, 0.0])),     # z = L, normal +z
        (np.array([0, 0, 0.0]), np.array([0, 0, 1.0]), np.array([0, 1, 0.0])),   # x = 0, normal -x
        (np.array([L, 0, 0.0]), np.array([0, 1, 0.0]), np.array([0, 0, 1.0])),   # x = L, normal +x
        (np.array([0, 0, 0.0]), np.array([1, 0, 0.0]), np.array([0, 0, 1.0])),   # y = 0, normal -y
        (np.array([0, L, 0.0]), np.array([0, 0, 1.0]), np.array([1, 0, 0.0])),   # y = L, normal +y
    ]
    for fi, (o, u, v) in enumerate(faces):
        for a in range(n):
            for b in range(n):
                p1 = o + u * g[a] + v * g[b]
                p2 = o + u * g[a + 1] + v * g[b]
                p3 = o + u * g[a + 1] + v * g[b + 1]
                p4 = o + u * g[a] + v * g[b + 1]
                conn.append([nid(p1), nid(p2), nid(p3), nid(p4)])
                face.append(fi)
    return np.array(nodes, dtype=np.float64), np.array(conn, dtype=np.int32), np.array(face)


def rsa_spheres(num: int, rng: np.random.Generator, lo, hi, radius_fn, min_dist_fn,
                max_tries: int = 2_000_000):
    """Seeded random sequential addition of `num` non-overlapping spheres whose
    centres lie in the box [lo, hi]^3; sphere k has radius radius_fn(k) and must
    keep centre distance >= min_dist_fn(r, radii placed so far)."""
    lo = np.broadcast_to(np.asarray(lo, dtype=np.float64), (3,))
    hi = np.broadcast_to(np.asarray(hi, dtype=np.float64), (3,))
    C = np.zeros((num, 3))
    R = np.zeros(num)
    k = 0
    tries = 0
    r = radius_fn(0)
    while k < num:
        tries += 1
        if tries > max_tries:
            raise RuntimeError(f"random sequential addition stalled at {k}/{num} spheres")
        c = lo + (hi - lo) * rng.random(3)
        if k:
            d = np.sqrt(((C[:k] - c) ** 2).sum(axis=1))
            if np.any(d < min_dist_fn(r, R[:k])):
                continue
        C[k] = c
        R[k] = r
        k += 1
        if k < num:
            r = radius_fn(k)
    return C, R


def cell_grid(n: int, lo, hi) -> np.ndarray:
    """Cell-centred n^3 sample grid over the box [lo, hi]^3 (x fastest)."""
    lo = np.broadcast_to(np.asarray(lo, dtype=np.float64), (3,))
    hi = np.broadcast_to(np.asarray(hi, dtype=np.float64), (3,))
    t = (np.arange(n) + 0.5) / n
    z, y, x = np.meshgrid(t, t, t, indexing="ij")
    p = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    return lo + p * (hi - lo)


def bounded_cube_case(n_face: int = 10, num: int = 64, radius: float = 0.05, grid: int = 32,
                      seed: int = 12345, E0: float = 70e9, nu0: float = 0.3, E1: float = 400e9,
                      nu1: float = 0.2, top_traction: float = 1.0) -> Case:
    """Unit cube with a Q4 boundary mesh (n_face^2 elements per face), bottom face
    fixed, uniform normal traction on the top face, other faces traction-free;
    `num` equal spheres placed by random sequential addition in [0.1, 0.9]^3 with
    centre distance >= 2.2 r; stresses sampled on a cell-centred grid^3."""
    nodes, conn, face = cube_mesh(n_face)
    NN, NE = len(nodes), len(conn)
    bottom_nodes = np.unique(conn[face == 0].ravel()) - 1
    bc = np.zeros((3 * NN, 2))
    bc[:, 0] = 1.0
    for j in bottom_nodes:
        bc[3 * j:3 * j + 3, 0] = 0.0
    tbc = np.zeros((NE, 24))
    tbc[:, :12] = 1.0
    tbc[face == 0, :12] = 0.0
    for e in np.nonzero(face == 1)[0]:
        tbc[e, 12 + 2::3] = top_traction
    rng = np.random.default_rng(seed)
    C, R = rsa_spheres(num, rng, 0.1, 0.9, lambda k: radius, lambda r, Rk: 2.2 * radius)
    pts = cell_grid(grid, 0.0, 1.0) if grid else np.zeros((0, 3))
    return Case(E0, nu0, E1, nu1, nodes, conn, bc, tbc, C, R, pts, None, "bounded_cube")


def farfield_case(num: int = 2000, r0: float = 0.012, vf: float = 0.15, grid: int = 64,
                  seed: int = 2024, E0: float = 70e9, nu0: float = 0.3, E1: float = 400e9,
                  nu1: float = 0.2, sigma33: float = 1.0) -> Case:
    """Boundary-free microstructure under a far-field uniaxial stress sigma33:
    `num` spheres with radius U[0.8, 1.2] r0, random sequential addition with a
    surface gap >= 0.1 r (r the larger radius of the pair), box side chosen from
    the target volume fraction `vf`; stresses on a cell-centred grid^3."""
    rng = np.random.default_rng(seed)
    radii = r0 * rng.uniform(0.8, 1.2, size=num)
    L = float((np.sum(4.0 / 3.0 * np.pi * radii ** 3) / vf) ** (1.0 / 3.0))
    C, R = rsa_spheres(num, rng, 1.2 * r0, L - 1.2 * r0, lambda k: radii[k],
                       lambda r, Rk: r + Rk + 0.1 * np.maximum(r, Rk))
    pts = cell_grid(grid, 0.0, L) if grid else np.zeros((0, 3))
    sig = np.array([0, 0, 0, 0, 0, sigma33], dtype=np.float64)
    return Case(E0, nu0, E1, nu1, np.zeros((0, 3)), np.zeros((0, 4), np.int32), np.zeros((0, 2)),
                np.zeros((0, 24)), C, R, pts, sig, "farfield")


def generated_case(num: int, r0: float, vf: float, seed: int, method: str = "mc", rlo: float = 0.8,
                   rhi: float = 1.2, gap: float = 0.1, grid: int = 0, E0: float = 70e9, nu0: float = 0.3,
                   E1: float = 400e9, nu1: float = 0.2, sigma33: float = 1.0) -> Case:
    """Boundary-free far-field case whose spheres come from the library's native generator
    (ibem_e3d_generate_spheres: "rsa" = random sequential addition inside the cube, "mc" =
    hard-sphere Monte Carlo with compression, which reaches 30% volume fraction).  The
    cube side L is returned in ``title`` as ``generated L=<side>``; stresses on grid^3."""
    import ctypes

    from . import GEN_MC, GEN_RSA, GenParams, check, lib
    p = GenParams(int(num), r0, rlo, rhi, vf, gap, GEN_MC if method == "mc" else GEN_RSA, int(seed), 0, 0)
    C = np.zeros((num, 3))
    R = np.zeros(num)
    side = ctypes.c_double(0.0)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    check(lib().ibem_e3d_generate_spheres(ctypes.byref(p), dp(C), dp(R), ctypes.byref(side)))
    L = side.value
    pts = cell_grid(grid, 0.0, L) if grid else np.zeros((0, 3))
    sig = np.array([0, 0, 0, 0, 0, sigma33], dtype=np.float64)
    return Case(E0, nu0, E1, nu1, np.zeros((0, 3)), np.zeros((0, 4), np.int32), np.zeros((0, 2)),
                np.zeros((0, 24)), C, R, pts, sig, f"generated L={L!r}")


def ellipsoid_case(num: int, a1: float = 0.008, vf: float = 0.15, seed: int = 31, grid: int = 0,
                   a2=(0.5, 1.0), a3=(0.25, 1.0), gap: float = 0.2, E0: float = 70e9, nu0: float = 0.3,
                   E1: float = 400e9, nu1: float = 0.2, sigma33: float = 1.0, max_tries: int = 0,
                   method: str = "rsa") -> Case:
    """Boundary-free far-field case of `num` ellipsoids from the library's generator
    (ibem_e3d_generate_ellipsoids): semi-axes a1, a1 U[a2], a1 U[a3], Haar-uniform
    orientations, random sequential addition ("rsa") or hard-ellipsoid Monte Carlo with
    compression ("mc", for volume fractions above ~20%) with the surfaces kept about
    gap * a3 apart, cube side from the volume fraction `vf`; stresses on a cell-centred
    grid^3.  `radius` holds the longest semi-axis (a bounding radius)."""
    import ctypes

    from . import GEN_MC, GEN_RSA, EllGenParams, check, lib
    p = EllGenParams(int(num), a1, a2[0], a2[1], a3[0], a3[1], vf, gap, int(seed), int(max_tries),
                     GEN_MC if method == "mc" else GEN_RSA, 0)
    C, A, Q = np.zeros((num, 3)), np.zeros((num, 3)), np.zeros((num, 4))
    side = ctypes.c_double(0.0)
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    check(lib().ibem_e3d_generate_ellipsoids(ctypes.byref(p), dp(C), dp(A), dp(Q), ctypes.byref(side)))
    L = side.value
    pts = cell_grid(grid, 0.0, L) if grid else np.zeros((0, 3))
    sig = np.array([0, 0, 0, 0, 0, sigma33], dtype=np.float64)
    return Case(E0, nu0, E1, nu1, np.zeros((0, 3)), np.zeros((0, 4), np.int32), np.zeros((0, 2)),
                np.zeros((0, 24)), C, A.max(axis=1), pts, sig, f"ellipsoids L={L!r}", A, Q)
