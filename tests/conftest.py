"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU."""
import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

PKG_NAME = "fast-cuda-gpu-dbscan_gb300"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (run with -m gpu)")
    config.addinivalue_line("markers", "slow: long-running full-size case")


def load_pkg():
    return importlib.import_module(PKG_NAME)


def load_datasets():
    return importlib.import_module(PKG_NAME + ".datasets")


@pytest.fixture(scope="session")
def gd():
    return load_pkg()


@pytest.fixture(scope="session")
def ds():
    return load_datasets()


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    return o


@pytest.fixture(scope="session")
def built_lib():
    """The CUDA library, built in-tree (the build itself needs no GPU)."""
    build = importlib.import_module(PKG_NAME + ".build")
    return build.build()


@pytest.fixture(scope="session")
def gpu_ctx(built_lib, gd):
    ctx = gd.Context(0)
    yield ctx
    ctx.close()


# ---- golden fixtures (labels of the reference's own R-tree DBSCAN) ---------
GOLDEN = os.path.join(ROOT, "tests", "golden", "rtree_golden.npz")


def golden_cases(names=None):
    """Yield (name, points, eps, minpts, labels) for every golden case."""
    import hashlib

    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden
    z = np.load(GOLDEN)
    all_names = sorted({k.split("/")[0] for k in z.files})
    for name in all_names:
        if names is not None and name not in names:
            continue
        key = f"{name}/points"
        pts = z[key] if key in z.files else make_golden.regenerate_points(name)
        dig = hashlib.sha256(np.ascontiguousarray(pts, dtype=np.float64).tobytes()).hexdigest()
        assert dig == z[f"{name}/digest"].item().decode(), f"golden points of {name} drifted"
        yield name, pts, float(z[f"{name}/eps"]), int(z[f"{name}/minpts"]), z[f"{name}/labels"]


def brute_dbscan(points, eps, minpts):
    """Pure-Python restatement of the reference's sequential expansion
    (cpu-dbscan/dbscan_rtree_exp.cpp:360-406) with a brute-force neighbour
    query, for small inputs (n of a few hundred) in 2D or 3D."""
    import numpy as np
    pts = np.asarray(points, dtype=np.float64)
    n, d = pts.shape
    e2 = eps * eps

    def nbrs(c):
        p = pts[c]
        lo, hi = p - eps, p + eps
        box = np.all((pts >= lo) & (pts <= hi), axis=1)
        dx = p[None, :] - pts
        s = dx[:, 0] * dx[:, 0]
        for k in range(1, d):
            s = s + dx[:, k] * dx[:, k]
        return np.nonzero(box & (s <= e2))[0].tolist()

    lab = [0] * n
    cluster = 0
    for i in range(n):
        if lab[i] != 0:
            continue
        nb = nbrs(i)
        if len(nb) < minpts:
            lab[i] = -1
            continue
        cluster += 1
        lab[i] = cluster
        j = 0
        while j < len(nb):
            q = nb[j]
            j += 1
            if q == i:
                continue
            if lab[q] == -1:
                lab[q] = cluster
                continue
            if lab[q] != 0:
                continue
            lab[q] = cluster
            more = nbrs(q)
            if len(more) >= minpts:
                nb.extend(more)
    out = np.array(lab, dtype=np.int32)
    return np.where(out == -1, -2, out - 1).astype(np.int32)
