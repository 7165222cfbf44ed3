"""Python host mirror of the gbdbscan C ABI (ctypes over libgbdbscan.so).

The reference is a compiled CUDA program with no Python surface; this module
exists so tests and benchmarks can drive the C ABI (include/gbdbscan.h) the
way a C/C++ caller would.  It adds no computation of its own: every call goes
to the CUDA library, and loading fails loudly when the library is missing.

Stages mirror the reference program (main.cu):
  import_dataset   ImportDataset            main.cu:469-498
  label_quality    cluster check            test-results/cluster-check.cpp:41-199
  Context.index_build   index construction  main.cu:166-338, indexing.cu
  Context.expand        expansion + merge   main.cu:369-403, dbscan.cu:25-387
  Context.get_result    GetDbscanResult     dbscan.cu:225-251
  Context.dbscan        all three
Labels: NOISE = -2 (common.h:8), clusters 0..K-1 ordered by smallest core index.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libgbdbscan.so")

GD_OK, GD_EINVAL, GD_ENOMEM, GD_ECUDA, GD_ERANGE, GD_ETIMEOUT, GD_EIO, GD_ENODEV, GD_ESTATE = range(9)
GD_PREC_FP64 = 0
GD_PREC_FP32_BAND = 1
NOISE = -2

_STATUS_NAMES = {0: "GD_OK", 1: "GD_EINVAL", 2: "GD_ENOMEM", 3: "GD_ECUDA", 4: "GD_ERANGE",
                 5: "GD_ETIMEOUT", 6: "GD_EIO", 7: "GD_ENODEV", 8: "GD_ESTATE"}


class GdError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{_STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class GdPoints(ctypes.Structure):
    _fields_ = [("coords", ctypes.c_void_p), ("n", ctypes.c_int64), ("dim", ctypes.c_int32),
                ("on_device", ctypes.c_int32)]


class GdInstance(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("dim", ctypes.c_int32), ("minpts", ctypes.c_int32),
                ("eps", ctypes.c_double)]


class GdStats(ctypes.Structure):
    _fields_ = [(name, ctypes.c_int64) for name in (
        "n_points", "n_clusters", "n_noise", "n_core", "n_border", "n_cells", "n_dense_cells",
        "tests_fp64", "tests_fp32", "band_retests", "asym_pairs", "grid_cells")] + [
        ("precision_used", ctypes.c_int32), ("key_bits", ctypes.c_int32),
        ("launches", ctypes.c_int32), ("reserved", ctypes.c_int32)] + [
        (name, ctypes.c_double) for name in (
            "ms_index", "ms_core", "ms_union", "ms_label", "ms_total", "ms_h2d", "ms_d2h")]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class GdTuning(ctypes.Structure):
    _fields_ = [("mult2d", ctypes.c_double), ("mult3d", ctypes.c_double),
                ("core_tests", ctypes.c_int32), ("link_tests", ctypes.c_int32),
                ("border_tests", ctypes.c_int32), ("reserved", ctypes.c_int32)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_ if name != "reserved"}


class GdServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("workers", ctypes.c_int32),
                ("max_batch", ctypes.c_int32), ("precision", ctypes.c_int32),
                ("hbm_budget_bytes", ctypes.c_int64)]


class GdRequestInfo(ctypes.Structure):
    _fields_ = [("n_clusters", ctypes.c_int64), ("status", ctypes.c_int32),
                ("batch_size", ctypes.c_int32), ("submit_ms", ctypes.c_double),
                ("start_ms", ctypes.c_double), ("done_ms", ctypes.c_double)]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class GdServerStats(ctypes.Structure):
    _fields_ = [(name, ctypes.c_int64) for name in (
        "submitted", "completed", "failed", "batches", "points", "max_batch_seen", "queued",
        "inflight_bytes")]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class GdLabelQuality(ctypes.Structure):
    _fields_ = [("score", ctypes.c_double), ("mismatch_loss", ctypes.c_double)] + [
        (name, ctypes.c_int64) for name in (
            "noise_mismatch", "noise_agree", "clusters_a", "clusters_b", "n")]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


_lib = None

# (name, restype, argtypes) of every entry point declared in include/gbdbscan.h
_P = ctypes.c_void_p
SIGNATURES = [
    ("gd_abi_version", ctypes.c_int32, []),
    ("gd_last_error", ctypes.c_char_p, []),
    ("gd_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("gd_ctx_create", ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(_P)]),
    ("gd_ctx_destroy", None, [_P]),
    ("gd_ctx_set_stream", ctypes.c_int, [_P, _P]),
    ("gd_ctx_set_precision", ctypes.c_int, [_P, ctypes.c_int32]),
    ("gd_ctx_set_cell_mult", ctypes.c_int, [_P, ctypes.c_double]),
    ("gd_ctx_set_cell_mults", ctypes.c_int, [_P, ctypes.c_double, ctypes.c_double]),
    ("gd_ctx_trim", ctypes.c_int, [_P]),
    ("gd_index_build", ctypes.c_int, [_P, ctypes.POINTER(GdPoints), ctypes.c_double]),
    ("gd_expand", ctypes.c_int, [_P, ctypes.c_int32]),
    ("gd_get_result", ctypes.c_int, [_P, _P, _P, ctypes.c_int32, ctypes.POINTER(ctypes.c_int64),
                                     ctypes.POINTER(ctypes.c_int64)]),
    ("gd_dbscan", ctypes.c_int, [_P, ctypes.POINTER(GdPoints), ctypes.c_double, ctypes.c_int32,
                                 _P, ctypes.POINTER(GdStats)]),
    ("gd_get_stats", ctypes.c_int, [_P, ctypes.POINTER(GdStats)]),
    ("gd_batch_dbscan", ctypes.c_int, [_P, ctypes.c_int32, _P, _P, ctypes.c_int32, _P, _P,
                                       ctypes.POINTER(GdStats)]),
    ("gd_ctx_set_graphs", ctypes.c_int, [_P, ctypes.c_int32]),
    ("gd_ctx_set_tuning", ctypes.c_int, [_P, ctypes.POINTER(GdTuning)]),
    ("gd_ctx_get_tuning", ctypes.c_int, [_P, ctypes.POINTER(GdTuning)]),
    ("gd_autotune", ctypes.c_int, [_P, ctypes.c_int32, _P, _P, ctypes.c_int32, ctypes.c_int32,
                                   ctypes.POINTER(GdTuning), ctypes.POINTER(ctypes.c_double)]),
    ("gd_server_create", ctypes.c_int, [ctypes.POINTER(GdServerConfig), ctypes.POINTER(_P)]),
    ("gd_server_destroy", None, [_P]),
    ("gd_server_submit", ctypes.c_int, [_P, ctypes.POINTER(GdInstance), _P, _P,
                                        ctypes.POINTER(ctypes.c_int64)]),
    ("gd_server_wait", ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_double,
                                      ctypes.POINTER(GdRequestInfo)]),
    ("gd_server_get_stats", ctypes.c_int, [_P, ctypes.POINTER(GdServerStats)]),
    ("gd_dbscan_noalloc", ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_int32, ctypes.c_double,
                                         ctypes.c_int32, ctypes.c_int32, _P,
                                         ctypes.POINTER(ctypes.c_int64), _P]),
    ("gd_import_dataset", ctypes.c_int, [ctypes.c_char_p, ctypes.c_int32, ctypes.c_int64,
                                         ctypes.POINTER(ctypes.POINTER(ctypes.c_double)),
                                         ctypes.POINTER(ctypes.c_int64)]),
    ("gd_write_labels", ctypes.c_int, [ctypes.c_char_p, _P, ctypes.c_int64]),
    ("gd_label_quality_compare", ctypes.c_int, [_P, _P, ctypes.c_int64, ctypes.c_int32,
                                                ctypes.POINTER(GdLabelQuality)]),
    ("gd_free", None, [_P]),
]


def load_library(path: str = LIB_PATH):
    """Load libgbdbscan.so (raises if it has not been built: there is no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it first (fast-cuda-gpu-dbscan_gb300/build.py)")
    lib = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(status: int) -> None:
    if status != GD_OK:
        lib = load_library()
        raise GdError(status, lib.gd_last_error().decode(errors="replace"))


def _instances(instances):
    """(gd_instance array, concatenated row-major float64 coordinates)."""
    desc = (GdInstance * max(len(instances), 1))()
    parts = []
    for i, (pts, eps, mp) in enumerate(instances):
        a = np.ascontiguousarray(pts, dtype=np.float64)
        desc[i].n = a.shape[0]
        desc[i].dim = a.shape[1]
        desc[i].minpts = int(mp)
        desc[i].eps = float(eps)
        parts.append(a.reshape(-1))
    coords = np.concatenate(parts) if parts else np.zeros(1)
    return desc, coords


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def import_dataset(path: str, dim: int, max_points: int = 0) -> np.ndarray:
    lib = load_library()
    out = ctypes.POINTER(ctypes.c_double)()
    n = ctypes.c_int64()
    _check(lib.gd_import_dataset(path.encode(), dim, max_points, ctypes.byref(out), ctypes.byref(n)))
    try:
        arr = np.ctypeslib.as_array(out, shape=(max(n.value, 1) * dim,))[: n.value * dim].copy()
    finally:
        lib.gd_free(ctypes.cast(out, ctypes.c_void_p))
    return arr.reshape(n.value, dim)


def label_quality(a, b, noise: int = NOISE) -> dict:
    """How far labelling ``b`` is from labelling ``a`` (the reference's cluster
    check): per point 0 when noise in exactly one, 1 when noise in both, else
    the Jaccard index of its two clusters; ``score`` is the mean.  Host code:
    needs no GPU."""
    la = np.ascontiguousarray(a, dtype=np.int32)
    lb = np.ascontiguousarray(b, dtype=np.int32)
    if la.shape != lb.shape or la.ndim != 1:
        raise ValueError("label_quality: a and b must be 1-D arrays of one length")
    q = GdLabelQuality()
    _check(load_library().gd_label_quality_compare(la.ctypes.data, lb.ctypes.data, la.shape[0],
                                                   int(noise), ctypes.byref(q)))
    return q.as_dict()


def write_labels(path: str, labels: np.ndarray) -> None:
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    _check(load_library().gd_write_labels(path.encode(), lab.ctypes.data, lab.shape[0]))


class Context:
    """One gbdbscan context (device memory pool + stream) on one GPU."""

    def __init__(self, device: int = 0, precision: int = GD_PREC_FP64, cell_mult: float = 0.0):
        self._lib = load_library()
        self._ctx = ctypes.c_void_p()
        _check(self._lib.gd_ctx_create(device, ctypes.byref(self._ctx)))
        self.set_precision(precision)
        if cell_mult:
            self.set_cell_mult(cell_mult)
        self._keep = None

    def close(self) -> None:
        if self._ctx:
            self._lib.gd_ctx_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_precision(self, precision: int) -> None:
        _check(self._lib.gd_ctx_set_precision(self._ctx, precision))

    def set_cell_mult(self, mult: float) -> None:
        _check(self._lib.gd_ctx_set_cell_mult(self._ctx, mult))

    def set_stream(self, stream_handle: int | None) -> None:
        _check(self._lib.gd_ctx_set_stream(self._ctx, stream_handle or None))

    def set_cell_mults(self, mult2d: float, mult3d: float) -> None:
        _check(self._lib.gd_ctx_set_cell_mults(self._ctx, mult2d, mult3d))

    def batch_dbscan(self, instances, with_stats: bool = False):
        """Cluster many independent instances in one run.

        ``instances``: list of (points (n, dim) float64, eps, minpts).  Returns a
        list of per-instance label arrays (cluster ids restart at 0 in each)."""
        desc, coords = _instances(instances)
        desc_list = list(desc)[: len(instances)]
        total = int(sum(d.n for d in desc_list))
        lab = np.empty(max(total, 1), dtype=np.int32)
        kc = np.zeros(max(len(instances), 1), dtype=np.int64)
        st = GdStats()
        _check(self._lib.gd_batch_dbscan(self._ctx, len(instances), desc, coords.ctypes.data, 0,
                                         lab.ctypes.data, kc.ctypes.data, ctypes.byref(st)))
        out, off = [], 0
        for d in desc_list:
            out.append(lab[off: off + d.n].copy())
            off += d.n
        if with_stats:
            return out, kc[: len(instances)].copy(), st.as_dict()
        return out

    def trim(self) -> None:
        _check(self._lib.gd_ctx_trim(self._ctx))

    def set_graphs(self, enable: bool) -> None:
        """Replay the expand launches as a CUDA graph on repeated gd_expand calls."""
        _check(self._lib.gd_ctx_set_graphs(self._ctx, 1 if enable else 0))

    # ---- tuning --------------------------------------------------------------
    def get_tuning(self) -> dict:
        t = GdTuning()
        _check(self._lib.gd_ctx_get_tuning(self._ctx, ctypes.byref(t)))
        return t.as_dict()

    def set_tuning(self, mult2d: float = 0.0, mult3d: float = 0.0, core_tests: int = 256,
                   link_tests: int = 48, border_tests: int = 160) -> None:
        t = GdTuning(mult2d, mult3d, core_tests, link_tests, border_tests, 0)
        _check(self._lib.gd_ctx_set_tuning(self._ctx, ctypes.byref(t)))

    def autotune(self, instances, repeats: int = 2) -> tuple[dict, float]:
        """Pick the fastest tuning for a sample of instances (list of (points,
        eps, minpts)); it is set on the context.  Returns (tuning, device ms)."""
        desc, coords = _instances(instances)
        t = GdTuning()
        ms = ctypes.c_double()
        _check(self._lib.gd_autotune(self._ctx, len(instances), desc, coords.ctypes.data, 0,
                                     int(repeats), ctypes.byref(t), ctypes.byref(ms)))
        return t.as_dict(), ms.value

    # ---- staged pipeline ---------------------------------------------------
    def _points(self, points):
        if _is_torch(points):
            import torch
            assert points.dtype == torch.float64 and points.is_contiguous() and points.dim() == 2
            on_dev = 1 if points.is_cuda else 0
            return GdPoints(points.data_ptr(), points.shape[0], points.shape[1], on_dev), points
        arr = np.ascontiguousarray(points, dtype=np.float64)
        if arr.ndim != 2:
            raise ValueError("points must be an (n, dim) array")
        return GdPoints(arr.ctypes.data, arr.shape[0], arr.shape[1], 0), arr

    def index_build(self, points, eps: float) -> None:
        gp, keep = self._points(points)
        self._keep = keep  # the library reads the points until expand() returns
        self._n = gp.n
        _check(self._lib.gd_index_build(self._ctx, ctypes.byref(gp), float(eps)))

    def expand(self, minpts: int) -> None:
        _check(self._lib.gd_expand(self._ctx, int(minpts)))

    def get_result(self, with_core: bool = False, out=None, core_out=None):
        """Labels (and core flags) in the caller's point order.

        ``out``/``core_out`` may be CUDA tensors (labels stay on the device)."""
        k = ctypes.c_int64()
        z = ctypes.c_int64()
        if out is not None and _is_torch(out) and out.is_cuda:
            cptr = core_out.data_ptr() if core_out is not None else None
            _check(self._lib.gd_get_result(self._ctx, out.data_ptr(), cptr, 1, ctypes.byref(k),
                                           ctypes.byref(z)))
            return (out, core_out) if with_core else out
        lab = np.empty(self._n, dtype=np.int32)
        core = np.empty(self._n, dtype=np.uint8) if with_core else None
        _check(self._lib.gd_get_result(self._ctx, lab.ctypes.data,
                                       core.ctypes.data if core is not None else None, 0,
                                       ctypes.byref(k), ctypes.byref(z)))
        return (lab, core.astype(bool)) if with_core else lab

    def stats(self) -> dict:
        st = GdStats()
        _check(self._lib.gd_get_stats(self._ctx, ctypes.byref(st)))
        return st.as_dict()

    def dbscan(self, points, eps: float, minpts: int, with_core: bool = False):
        """Exact DBSCAN; returns labels (numpy int32, or a CUDA tensor for CUDA input)."""
        if _is_torch(points) and points.is_cuda:
            import torch
            out = torch.empty(points.shape[0], dtype=torch.int32, device=points.device)
            core = torch.empty(points.shape[0], dtype=torch.uint8, device=points.device) \
                if with_core else None
            self.index_build(points, eps)
            self.expand(minpts)
            return self.get_result(with_core, out=out, core_out=core)
        self.index_build(points, eps)
        self.expand(minpts)
        return self.get_result(with_core)

    def dbscan_fused(self, points, eps: float, minpts: int) -> tuple[np.ndarray, dict]:
        """The one-call entry point gd_dbscan (host arrays)."""
        gp, keep = self._points(points)
        lab = np.empty(gp.n, dtype=np.int32)
        st = GdStats()
        _check(self._lib.gd_dbscan(self._ctx, ctypes.byref(gp), float(eps), int(minpts),
                                   lab.ctypes.data, ctypes.byref(st)))
        return lab, st.as_dict()


class Server:
    """Request server with continuous batching (gd_server_* in the C ABI).

    ``submit(points, eps, minpts)`` queues one clustering request and returns its
    id; ``wait(id)`` returns (labels, info) once it has run.  Worker threads in
    the library each own a context and CUDA stream and cluster every admissible
    queued request together; each request's labels equal those of
    ``Context.dbscan`` on that request alone."""

    def __init__(self, device: int = 0, workers: int = 2, max_batch: int = 1024,
                 precision: int = GD_PREC_FP64, hbm_budget_bytes: int = 64 << 30):
        self._lib = load_library()
        cfg = GdServerConfig(device, workers, max_batch, precision, hbm_budget_bytes)
        h = ctypes.c_void_p()
        _check(self._lib.gd_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._srv = h
        self._pending = {}  # request id -> (points, labels) kept alive until waited for

    def close(self) -> None:
        if getattr(self, "_srv", None):
            self._lib.gd_server_destroy(self._srv)
            self._srv = None
            self._pending.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, points, eps: float, minpts: int) -> int:
        a = np.ascontiguousarray(points, dtype=np.float64)
        if a.ndim != 2:
            raise ValueError("points must be (n, dim)")
        lab = np.empty(max(a.shape[0], 1), dtype=np.int32)
        inst = GdInstance(a.shape[0], a.shape[1], int(minpts), float(eps))
        rid = ctypes.c_int64()
        _check(self._lib.gd_server_submit(self._srv, ctypes.byref(inst), a.ctypes.data,
                                          lab.ctypes.data, ctypes.byref(rid)))
        self._pending[rid.value] = (a, lab)
        return rid.value

    def wait(self, request_id: int, timeout_ms: float = -1.0):
        info = GdRequestInfo()
        st = self._lib.gd_server_wait(self._srv, int(request_id), float(timeout_ms),
                                      ctypes.byref(info))
        if st == GD_ETIMEOUT:
            _check(st)  # still running: keep its buffers
        entry = self._pending.pop(int(request_id), None)
        _check(st)
        a, lab = entry
        return lab[: a.shape[0]].copy(), info.as_dict()

    def stats(self) -> dict:
        st = GdServerStats()
        _check(self._lib.gd_server_get_stats(self._srv, ctypes.byref(st)))
        return st.as_dict()
