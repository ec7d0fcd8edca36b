"""Regenerates the golden fixtures of this directory from the reference itself.

Needs the reference sources (IBEM_REFERENCE_DIR, or a directory named `reference`
beside the repository): the reference's own elastic-3D translation units are
compiled by `make -C oracle ref` into oracle/_ref/ibem_ref and run here.  Outputs
(committed):

  kat_reference.npz      D_40..D_62, IGreen_01/11/21 and Green_01..04 at three points
                         (outside, near the surface, inside), materials E0 nu0 E1 nu1
  example_reference.npz  the reference's examples/elastic3D_spherical inputs, its
                         X, U, T and stresses as computed here, and the 103 comparable
                         rows of its "stress ground truth.txt"
  tiny_reference.npz     a 2-sphere bounded cube (2 x 2 elements per face), HMAT,
                         GMAT, b, X, U, T and stresses from the reference (78 unknowns;
                         A is HMAT/GMAT after ApplyBC and is rebuilt from them)
  cube64_reference.npz   the bounded unit cube of 6 x 10 x 10 Q4 elements per face with
                         64 spheres (r = 0.05, seed 12345; 600 elements, N = 6,798 at 78
                         unknowns per sphere): the reference's X and its stresses at a
                         seeded 1,024-point subset of the 32^3 cell-centred grid, and the
                         oracle's X and stresses for the 24-unknown truncation (N = 3,342,
                         full-pivot LU); no matrices (N^2 doubles).  Slow: about ten
                         minutes of the reference on 8 cores.
  python make_golden.py [kat] [example] [tiny] [cube64]   (default: all)
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from ibemproject_gb300 import cases  # noqa: E402
import oracle  # noqa: E402

REF = oracle.reference_dir()


def run_ref(workdir, *args):
    subprocess.run([oracle.REF_BIN, *args], check=True, stdout=subprocess.DEVNULL, cwd=workdir)


def kat():
    pts = np.array([[0.071, -0.032, 0.055, 0.05],    # outside
                    [0.0301, 0.0402, 0.0, 0.05],     # just outside the surface
                    [0.012, -0.02, 0.015, 0.05]])    # inside
    mat = np.array([70e9, 0.3, 400e9, 0.2])
    with tempfile.TemporaryDirectory() as d:
        np.save(os.path.join(d, "kat_in.npy"), pts)
        np.save(os.path.join(d, "kat_mat.npy"), mat)
        run_ref(d, "kat", d)
        out = {k: np.load(os.path.join(d, f"kat_{k}.npy")) for k in
               ["D40", "D50", "D60", "D41", "D51", "D61", "D42", "D52", "D62", "IG0", "IG1", "IG2",
                "G1", "G2", "G3", "G4"]}
    np.savez_compressed(os.path.join(HERE, "kat_reference.npz"), points=pts, mat=mat, **out)


def case_arrays(c):
    return dict(E0=c.E0, nu0=c.nu0, E1=c.E1, nu1=c.nu1, nodes=c.nodes, conn=c.conn, bc=c.bc, tbc=c.tbc,
                centers=c.centers, radius=c.radius, points=c.points)


def example():
    src = os.path.join(REF, "examples", "elastic3D_spherical")
    c = cases.read_case(src)
    with tempfile.TemporaryDirectory() as d:
        for f in ("BEM.txt", "position.txt", "postprocess.txt"):
            shutil.copy(os.path.join(src, f), d)
        run_ref(d, "run", d)
        X = np.load(os.path.join(d, "X.npy"))
        U = np.load(os.path.join(d, "U.npy"))
        T = np.load(os.path.join(d, "T.npy"))
        S = np.load(os.path.join(d, "stress.npy"))
    gt = np.loadtxt(os.path.join(src, "stress ground truth.txt"))[:c.nump]
    np.savez_compressed(os.path.join(HERE, "example_reference.npz"), X=X, U=U, T=T, stress=S,
                        ground_truth=gt, **case_arrays(c))


def tiny():
    c = cases.bounded_cube_case(n_face=2, num=2, radius=0.12, grid=3, seed=7, top_traction=1e4)
    with tempfile.TemporaryDirectory() as d:
        cases.write_case(d, c)
        run_ref(d, "run", d)
        out = {k: np.load(os.path.join(d, f"{k}.npy")) for k in ["HMAT", "GMAT", "b", "X", "U", "T", "stress"]}
    np.savez_compressed(os.path.join(HERE, "tiny_reference.npz"), **out, **case_arrays(c))


CUBE64_SUBSET_SEED = 2025


def cube64_subset(nump):
    """The seeded 1,024-point subset of the 32^3 grid that the cube64 fixture samples."""
    return np.sort(np.random.default_rng(CUBE64_SUBSET_SEED).choice(nump, 1024, replace=False))


def cube64():
    c = cases.bounded_cube_case(n_face=10, num=64, radius=0.05, grid=32, seed=12345)
    idx = cube64_subset(c.nump)
    c.points = c.points[idx]
    with tempfile.TemporaryDirectory() as d:
        cases.write_case(d, c)
        run_ref(d, "run", d, "--no-matrices")
        X78 = np.load(os.path.join(d, "X.npy"))
        S78 = np.load(os.path.join(d, "stress.npy"))
        timings = open(os.path.join(d, "timings.txt")).read()
    # the 24-unknown truncation: the same entries restricted to orders 0-1, solved by the
    # oracle's full-pivot LU (the reference's fullPivLu algorithm)
    m = oracle.mat(c.E0, c.nu0, c.E1, c.nu1)
    H, G = oracle.assemble(c, 24, m)
    A, b, tcol, _ = oracle.apply_bc(c, H, G)
    X24 = oracle.solve_fullpiv(A, b)
    U24, T24 = oracle.get_ut(c, tcol, X24)
    S24 = oracle.post(c, 24, X24[3 * c.NN:], U24, T24, m=m)
    np.savez_compressed(os.path.join(HERE, "cube64_reference.npz"), X78=X78, stress78=S78, X24=X24, stress24=S24,
                        subset=idx, centers=c.centers, radius=c.radius, points=c.points,
                        ref_timings=np.array(timings))


if __name__ == "__main__":
    if oracle.build_ref() is None:
        sys.exit("reference sources not found")
    which = sys.argv[1:] or ["kat", "example", "tiny", "cube64"]
    for name in which:
        {"kat": kat, "example": example, "tiny": tiny, "cube64": cube64}[name]()
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
