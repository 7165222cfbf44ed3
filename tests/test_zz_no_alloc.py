"""gd_dbscan_noalloc: the entry point for callers that cannot allocate device
memory -- loops that reserve all their device memory at start-up (an allocation
can block, and cudaFree waits for the whole device) and plug-ins whose host
process owns the GPU's memory.

It runs the same kernels as gd_dbscan out of one fixed static device array, so
its labels must equal gd_dbscan's bit for bit (integer labels: no tolerance).
This file is collected last on purpose: it must pass alone in a fresh process
and after every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, pts_t, eps, minpts, precision, out_t):
    k = ctypes.c_int64(-1)
    st = lib.gd_dbscan_noalloc(pts_t.data_ptr(), pts_t.shape[0], pts_t.shape[1], float(eps),
                               int(minpts), int(precision), out_t.data_ptr(), ctypes.byref(k),
                               None)
    return st, k.value


def _cases(ds):
    a = ds.blobs2d_100k(seed=5, scale=0.25)                       # 25,000 points, 2D
    b = ds.aniso3d_20m(seed=6, scale=0.0015)                      # 30,000 points, 3D
    rng = np.random.default_rng(9)
    far = np.concatenate([c + rng.normal(0, 0.2, (2000, 2))       # sparse grid (hash path)
                          for c in rng.uniform(-1e4, 1e4, (5, 2))])
    return [(a.points, a.eps, a.minpts), (b.points, b.eps, b.minpts), (far, 0.05, 6)]


def test_noalloc_matches_gd_dbscan_on_consecutive_calls(built_lib, gd, ds):
    import torch
    lib = gd.load_library()
    with gd.Context(0) as ctx:
        for precision in (gd.GD_PREC_FP64, gd.GD_PREC_FP32_BAND):
            ctx.set_precision(precision)
            # two calls in a row on different inputs, each checked against gd_dbscan
            for pts, eps, mp in _cases(ds):
                assert pts.shape[0] <= 32768
                want, st = ctx.dbscan_fused(pts, eps, mp)
                t = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
                out = torch.full((pts.shape[0],), 12345, dtype=torch.int32, device="cuda")
                status, k = _noalloc(lib, t, eps, mp, precision, out)
                assert status == 0, lib.gd_last_error().decode()
                assert np.array_equal(out.cpu().numpy(), want)
                assert k == st["n_clusters"]


def test_noalloc_repeat_allocates_nothing(built_lib, gd, ds):
    import torch
    lib = gd.load_library()
    pts, eps, mp = _cases(ds)[0]
    t = torch.from_numpy(np.ascontiguousarray(pts)).cuda()
    out1 = torch.empty(pts.shape[0], dtype=torch.int32, device="cuda")
    out2 = torch.empty(pts.shape[0], dtype=torch.int32, device="cuda")
    assert _noalloc(lib, t, eps, mp, 0, out1)[0] == 0     # first call: address set-up
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    assert _noalloc(lib, t, eps, mp, 0, out2)[0] == 0
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    assert torch.equal(out1, out2)


def test_noalloc_rejects_oversize_and_bad_args(built_lib, gd):
    import torch
    lib = gd.load_library()
    big = torch.zeros((32769, 2), dtype=torch.float64, device="cuda")
    out = torch.empty(32769, dtype=torch.int32, device="cuda")
    st, _ = _noalloc(lib, big, 1.0, 2, 0, out)
    assert st == 4 and b"32768" in lib.gd_last_error()
    small = torch.zeros((8, 2), dtype=torch.float64, device="cuda")
    assert _noalloc(lib, small, 0.0, 2, 0, out)[0] == 1
    assert _noalloc(lib, small, 1.0, 0, 0, out)[0] == 1
    nan = torch.tensor([[0.0, float("nan")], [1.0, 1.0]], dtype=torch.float64, device="cuda")
    assert _noalloc(lib, nan, 1.0, 1, 0, out)[0] == 1
