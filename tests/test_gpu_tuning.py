"""Tuning (gd_ctx_set_tuning, gd_autotune): cell multipliers and per-thread test
budgets change speed, never labels.  Every tuning must give the oracle's
labels; the autotuner must return a valid tuning and leave it on the context."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TUNINGS = [
    dict(),                                                     # defaults
    dict(mult2d=0.7, mult3d=0.577, core_tests=256, link_tests=48, border_tests=160),
    dict(mult2d=0.55, mult3d=0.53, core_tests=0, link_tests=0, border_tests=0),   # all to warps
    dict(mult2d=0.6, mult3d=0.55, core_tests=4096, link_tests=4096, border_tests=4096),
    dict(core_tests=1, link_tests=1, border_tests=1),
]


def _sample(seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = int(rng.choice([2, 3]))
        n = int(rng.integers(50, 3000))
        k = int(rng.integers(1, 5))
        c = rng.uniform(0, 20, (k, d))
        pts = np.concatenate([c[rng.integers(0, k, n)] + rng.normal(0, 0.8, (n, d)),
                              rng.uniform(0, 20, (n // 10 + 1, d))])
        out.append((pts, float(rng.uniform(0.3, 0.9)), int(rng.integers(3, 15))))
    return out


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("ti", range(len(TUNINGS)))
def test_every_tuning_gives_oracle_labels(gpu_ctx, oracle, prec, ti):
    insts = _sample(7, 24)
    gpu_ctx.set_precision(prec)
    gpu_ctx.set_tuning(**TUNINGS[ti])
    try:
        labels = gpu_ctx.batch_dbscan(insts)
        for (p, e, m), lab in zip(insts, labels):
            assert np.array_equal(lab, oracle.oracle_dbscan(p, e, m)[0])
        p, e, m = insts[0]
        assert np.array_equal(gpu_ctx.dbscan(p, e, m), oracle.oracle_dbscan(p, e, m)[0])
    finally:
        gpu_ctx.set_tuning()


def test_tuning_validation_and_roundtrip(gpu_ctx, gd):
    gpu_ctx.set_tuning(mult2d=0.6, mult3d=0.55, core_tests=100, link_tests=20, border_tests=30)
    t = gpu_ctx.get_tuning()
    assert t["mult2d"] == 0.6 and t["mult3d"] == 0.55
    assert (t["core_tests"], t["link_tests"], t["border_tests"]) == (100, 20, 30)
    for bad in [dict(mult2d=0.75), dict(mult3d=0.6), dict(core_tests=-1),
                dict(border_tests=70000)]:
        with pytest.raises(gd.GdError) as e:
            gpu_ctx.set_tuning(**bad)
        assert e.value.status == 1
    gpu_ctx.set_tuning()
    assert gpu_ctx.get_tuning()["core_tests"] == 256


def test_autotune_sets_a_valid_tuning(gpu_ctx, oracle):
    insts = _sample(9, 16)
    t, ms = gpu_ctx.autotune(insts, repeats=1)
    try:
        assert ms > 0
        assert 0.5 < t["mult2d"] <= 0.7072 and 0.5 < t["mult3d"] <= 0.5774
        assert gpu_ctx.get_tuning() == t
        labels = gpu_ctx.batch_dbscan(insts)
        for (p, e, m), lab in zip(insts, labels):
            assert np.array_equal(lab, oracle.oracle_dbscan(p, e, m)[0])
    finally:
        gpu_ctx.set_tuning()


@pytest.mark.parametrize("graphs", [True, False])
def test_minpts_sweep_replays_the_expand_graph(gpu_ctx, ds, oracle, graphs):
    """gd_expand on one index with several minpts (the second call captures the
    expand launches, later ones replay them): every result is the oracle's."""
    inst = ds.zipf2d_10m(seed=5, scale=0.01)
    gpu_ctx.set_graphs(graphs)
    try:
        for prec in (0, 1):
            gpu_ctx.set_precision(prec)
            gpu_ctx.index_build(inst.points, inst.eps)
            for mp in (8, 4, 16, 8, 30, 2):
                gpu_ctx.expand(mp)
                lab = gpu_ctx.get_result()
                assert np.array_equal(lab, oracle.oracle_dbscan(inst.points, inst.eps, mp)[0]), mp
                st = gpu_ctx.stats()
                assert st["ms_core"] > 0 and st["ms_union"] >= 0
        # a tuning change drops the graph; the next sweep recaptures
        gpu_ctx.set_tuning(core_tests=64)
        gpu_ctx.index_build(inst.points, inst.eps)
        for mp in (5, 9, 5):
            gpu_ctx.expand(mp)
            assert np.array_equal(gpu_ctx.get_result(),
                                  oracle.oracle_dbscan(inst.points, inst.eps, mp)[0])
    finally:
        gpu_ctx.set_tuning()
        gpu_ctx.set_graphs(True)
