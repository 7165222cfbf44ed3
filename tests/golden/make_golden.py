"""Generate golden label fixtures from the reference's own exact CPU DBSCAN.

Runs the reference's cpu-dbscan/dbscan_rtree_exp.cpp (compiled from the
reference checkout by oracle/build.py into oracle/_ref/) on seeded inputs and
stores its labels (mapped to NOISE=-2, clusters 0..K-1) in rtree_golden.npz.
The reference program is 2D only, so every golden case is 2D.

    python tests/golden/make_golden.py        (needs the reference checkout)

Cases:
  ex_txt           the reference's own fixture test-datasets/ex.txt with its
                   shipped common.h (EPS 1.5, MINPTS 3)
  tiny_*           the 2D hand-made edge cases of datasets.tiny_cases()
  asym_xy, asym_yx the one-directional neighbour pair p=(1e-20,0), q=(-0.3,0),
                   eps=0.3, in both point orders (one cluster vs two)
  rand_*           seeded random 2D sets: integer lattices (exact d^2 == eps^2
                   ties) and Gaussian mixtures at mixed scales
  c1_seed0         the 100,000-point 2D blob set
Points are stored for the small cases; the Gaussian ones and c1_seed0 keep only
a SHA-256 digest of their points and are regenerated by regenerate_points().
"""
from __future__ import annotations

import hashlib
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

ds = importlib.import_module("fast-cuda-gpu-dbscan_gb300.datasets")
REF_EX = os.path.join(O._build.REF_ROOT, "test-datasets", "ex.txt")


def digest(points: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(points, dtype=np.float64).tobytes()).hexdigest()


def random_cases():
    rng = np.random.Generator(np.random.PCG64(20251203))
    out = []
    for t in range(24):
        n = int(rng.integers(5, 600))
        side = int(rng.integers(3, 40))
        pts = rng.integers(0, side, size=(n, 2)).astype(np.float64)
        eps = float(rng.choice([1.0, 2.0, 5.0, 1.5, np.sqrt(2.0), 2.5]))
        out.append((f"rand_lattice_{t}", pts, eps, int(rng.integers(1, 12))))
    for t in range(24):
        n = int(rng.integers(5, 4000))
        pts = rng.normal(0, rng.uniform(0.2, 3), size=(n, 2)) * 10 ** rng.uniform(-3, 3)
        pts += rng.uniform(-5, 5, size=2) * 10 ** rng.uniform(-3, 3)
        eps = float(np.std(pts) * rng.uniform(0.02, 0.3))
        out.append((f"rand_gauss_{t}", pts, eps, int(rng.integers(1, 20))))
    return out


def regenerate_points(name: str) -> np.ndarray:
    """Points of a golden case whose points are not stored in the fixture."""
    if name == "c1_seed0":
        return ds.blobs2d_100k(seed=0).points
    for cname, pts, _eps, _mp in random_cases():
        if cname == name:
            return pts
    raise KeyError(name)


def main() -> None:
    if not O.ref_available():
        sys.exit("reference checkout not found; cannot regenerate golden fixtures")
    store = {}

    def add(name, pts, eps, minpts, keep_points=True):
        lab, k = O.ref_rtree_dbscan(pts, eps, minpts)
        store[f"{name}/eps"] = np.float64(eps)
        store[f"{name}/minpts"] = np.int32(minpts)
        store[f"{name}/labels"] = lab
        store[f"{name}/digest"] = np.bytes_(digest(pts))
        if keep_points:
            store[f"{name}/points"] = np.ascontiguousarray(pts, dtype=np.float64)
        print(f"{name:24s} n={len(pts):7d} clusters={k:5d} noise={(lab == -2).sum()}")

    ex = np.loadtxt(REF_EX, delimiter=",", dtype=np.float64)
    add("ex_txt", ex, 1.5, 3)
    for inst in ds.tiny_cases():
        if inst.dim == 2 and inst.name != "ex_txt":
            add(f"tiny_{inst.name}", inst.points, inst.eps, inst.minpts)
    X = [[1e-20, 0.0], [0.1, 0.0], [0.2, 0.0]]
    Y = [[-0.3, 0.0], [-0.4, 0.0], [-0.5, 0.0]]
    add("asym_xy", np.array(X + Y), 0.3, 3)
    add("asym_yx", np.array(Y + X), 0.3, 3)
    for name, pts, eps, mp in random_cases():
        add(name, pts, eps, mp, keep_points=name.startswith("rand_lattice"))
    c1 = ds.blobs2d_100k(seed=0)
    add("c1_seed0", c1.points, c1.eps, c1.minpts, keep_points=False)
    np.savez_compressed(os.path.join(HERE, "rtree_golden.npz"), **store)


if __name__ == "__main__":
    main()
