"""Request server (gd_server_*): continuous batching over gd_batch_dbscan.

Every request's labels must be the same whether it ran alone or in a batch
with other requests, and equal the oracle's (bit-exact).  The admission
budget and the batch limit must hold."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(seed, count, lo=30, hi=6000):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = int(rng.choice([2, 3]))
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        k = int(rng.integers(1, 6))
        centres = rng.uniform(0, 20, (k, d))
        pts = np.concatenate([centres[rng.integers(0, k, n)] + rng.normal(0, 0.7, (n, d)),
                              rng.uniform(0, 20, (n // 8 + 1, d))])
        scale = 10 ** rng.uniform(-1, 1)
        out.append((pts * scale, float(rng.uniform(0.3, 1.0) * scale), int(rng.integers(2, 12))))
    return out


@pytest.mark.parametrize("prec", [0, 1])
def test_server_results_equal_alone_and_in_the_mix(gd, gpu_ctx, oracle, prec):
    reqs = _requests(11 + prec, 120)
    gpu_ctx.set_precision(prec)
    alone = [gpu_ctx.dbscan(p, e, m) for p, e, m in reqs]
    with gd.Server(0, workers=2, max_batch=64, precision=prec) as srv:
        # submit from several threads at once so batches form from a mixed queue
        ids = [None] * len(reqs)

        def submit(part):
            for i in part:
                ids[i] = srv.submit(*reqs[i])

        th = [threading.Thread(target=submit, args=(range(t, len(reqs), 4),)) for t in range(4)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        got = [srv.wait(i) for i in ids]
        stats = srv.stats()
    assert stats["completed"] == len(reqs) and stats["failed"] == 0
    assert stats["batches"] < len(reqs)        # requests were batched together
    assert max(info["batch_size"] for _, info in got) > 1
    for (p, e, m), want, (lab, info) in zip(reqs, alone, got):
        assert np.array_equal(lab, want)
        assert info["status"] == 0
        assert info["n_clusters"] == (want.max() + 1 if (want >= 0).any() else 0)
        assert info["submit_ms"] <= info["start_ms"] <= info["done_ms"]
    for (p, e, m), (lab, _) in list(zip(reqs, got))[:20]:
        assert np.array_equal(lab, oracle.oracle_dbscan(p, e, m)[0])


def test_server_budget_and_batch_limit(gd, gpu_ctx):
    reqs = _requests(3, 40, lo=200, hi=2000)
    want = [gpu_ctx.dbscan(p, e, m) for p, e, m in reqs]
    # a budget below every request's estimate: each runs alone, one at a time
    with gd.Server(0, workers=2, max_batch=64, hbm_budget_bytes=1 << 10) as srv:
        ids = [srv.submit(*r) for r in reqs]
        got = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st["max_batch_seen"] == 1 and st["batches"] == len(reqs)
    assert all(np.array_equal(l, w) for (l, _), w in zip(got, want))
    # no budget limit, at most 8 requests per batch
    with gd.Server(0, workers=1, max_batch=8) as srv:
        ids = [srv.submit(*r) for r in reqs]
        got = [srv.wait(i) for i in ids]
        st = srv.stats()
    assert st["max_batch_seen"] <= 8
    assert all(info["batch_size"] <= 8 for _, info in got)
    assert all(np.array_equal(l, w) for (l, _), w in zip(got, want))


def test_server_edge_requests_and_errors(gd, gpu_ctx):
    with gd.Server(0, workers=1) as srv:
        ok = srv.submit(np.zeros((0, 2)), 1.0, 3)
        one = srv.submit(np.array([[1.0, 2.0, 3.0]]), 0.5, 1)
        lab, info = srv.wait(ok)
        assert lab.shape == (0,) and info["n_clusters"] == 0
        lab, info = srv.wait(one)
        assert lab.tolist() == [0] and info["n_clusters"] == 1
        for bad in [(np.zeros((4, 2)), 0.0, 2), (np.zeros((4, 2)), 1.0, 0),
                    (np.array([[0.0, np.nan]]), 1.0, 1), (np.zeros((4, 4)), 1.0, 2)]:
            with pytest.raises(gd.GdError) as e:
                srv.submit(*bad)
            assert e.value.status == 1
        with pytest.raises(gd.GdError) as e:
            srv.wait(10 ** 9)                  # unknown request id
        assert e.value.status == 1
        assert srv.stats()["failed"] == 0
