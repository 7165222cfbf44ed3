"""ctypes access to the checker libraries (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline legs may import
this module.  Label convention of every function here: NOISE = -2 (common.h:8),
clusters 0..K-1 numbered by their smallest core point index.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

_oracle = None
_ref = None


def _load_oracle():
    global _oracle
    if _oracle is None:
        lib = ctypes.CDLL(_build.build_oracle())
        lib.gd_oracle_dbscan.restype = ctypes.c_int
        lib.gd_oracle_dbscan.argtypes = [
            ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double, ctypes.c_int,
            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.gd_oracle_pred.restype = ctypes.c_int
        lib.gd_oracle_pred.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_double]
        _oracle = lib
    return _oracle


def oracle_dbscan(points: np.ndarray, eps: float, minpts: int, nthreads: int = 0):
    """Exact DBSCAN on the CPU. Returns (labels int32, is_core bool, counters dict)."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    n, d = pts.shape
    labels = np.empty(n, dtype=np.int32)
    core = np.empty(n, dtype=np.uint8)
    cnt = np.zeros(8, dtype=np.int64)
    rc = _load_oracle().gd_oracle_dbscan(
        pts.ctypes.data, n, d, float(eps), int(minpts), int(nthreads),
        labels.ctypes.data, core.ctypes.data, cnt.ctypes.data)
    if rc != 0:
        raise ValueError(f"oracle rejected the input (code {rc})")
    keys = ["clusters", "noise", "core", "border", "asym_pairs", "sequential",
            "pred_tests", "cells"]
    return labels, core.astype(bool), dict(zip(keys, (int(v) for v in cnt)))


def oracle_pred(c, q, eps: float) -> bool:
    c = np.ascontiguousarray(c, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    return bool(_load_oracle().gd_oracle_pred(c.ctypes.data, q.ctypes.data, c.shape[0],
                                              float(eps)))


def ref_available() -> bool:
    return os.path.exists(_build.REF_RTREE_SO) or _build.build_ref() is not None


def ref_rtree_dbscan(points: np.ndarray, eps: float, minpts: int):
    """The reference's own R-tree DBSCAN (2D only). Labels mapped to -2 / 0..K-1."""
    global _ref
    if _ref is None:
        path = _build.REF_RTREE_SO if os.path.exists(_build.REF_RTREE_SO) else _build.build_ref()
        if path is None:
            raise RuntimeError("reference R-tree build unavailable")
        lib = ctypes.CDLL(path)
        lib.gd_ref_rtree_dbscan.restype = ctypes.c_int
        lib.gd_ref_rtree_dbscan.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                            ctypes.c_int, ctypes.c_void_p]
        _ref = lib
    pts = np.ascontiguousarray(points, dtype=np.float64)
    assert pts.shape[1] == 2, "the reference R-tree DBSCAN is 2D only"
    n = pts.shape[0]
    raw = np.empty(n, dtype=np.int32)
    k = _ref.gd_ref_rtree_dbscan(pts.ctypes.data, n, float(eps), int(minpts), raw.ctypes.data)
    lab = np.where(raw == -1, -2, raw - 1).astype(np.int32)
    return lab, int(k)


_mc = None


def ref_multicore_dbscan(points: np.ndarray, eps: float, minpts: int, threads: int = 16) -> int:
    """The reference's multicore CPU DBSCAN (2D, O(n^2) brute force, float32
    sqrt test, self excluded from the count) on these points; returns the
    number of clusters it reports.  For timing: its semantics differ from the
    exact DBSCAN, so its clusters are not compared with anything."""
    global _mc
    if _mc is None:
        path = (_build.REF_MULTICORE_SO if os.path.exists(_build.REF_MULTICORE_SO)
                else _build.build_ref_multicore())
        if path is None:
            raise RuntimeError("reference multicore build unavailable")
        lib = ctypes.CDLL(path)
        lib.gd_ref_multicore_dbscan.restype = ctypes.c_int
        lib.gd_ref_multicore_dbscan.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double,
                                                ctypes.c_int, ctypes.c_int]
        _mc = lib
    pts = np.ascontiguousarray(points, dtype=np.float64)
    assert pts.shape[1] == 2, "the reference multicore DBSCAN is 2D only"
    return int(_mc.gd_ref_multicore_dbscan(pts.ctypes.data, pts.shape[0], float(eps),
                                           int(minpts), int(threads)))
