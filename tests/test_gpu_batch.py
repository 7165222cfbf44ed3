"""Batched DBSCAN (gd_batch_dbscan): many independent instances, each with its
own eps, minpts and dimension, clustered in one run.  Every instance's labels
must equal the oracle's for that instance alone (bit-exact, ids restarting at 0
in every instance)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mixed_instances(seed, count, lo=20, hi=4000):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        d = int(rng.choice([2, 3]))
        n = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        k = int(rng.integers(1, 8))
        centres = rng.uniform(0, 30, (k, d))
        pts = np.concatenate([centres[rng.integers(0, k, n)] + rng.normal(0, rng.uniform(0.3, 2), (n, d)),
                              rng.uniform(0, 30, (max(1, n // 10), d))])
        scale = 10 ** rng.uniform(-2, 2)
        pts = pts * scale + rng.uniform(-100, 100)
        eps = float(rng.uniform(0.3, 1.5) * scale)
        out.append((pts, eps, int(rng.integers(2, 20))))
    return out


@pytest.mark.parametrize("prec", [0, 1])
def test_batch_matches_oracle_per_instance(gpu_ctx, oracle, prec):
    insts = _mixed_instances(5 + prec, 60)
    gpu_ctx.set_precision(prec)
    labels, counts, st = gpu_ctx.batch_dbscan(insts, with_stats=True)
    assert st["n_points"] == sum(p.shape[0] for p, _, _ in insts)
    for (pts, eps, mp), lab, k in zip(insts, labels, counts):
        want, _, c = oracle.oracle_dbscan(pts, eps, mp)
        assert np.array_equal(lab, want)
        assert k == c["clusters"]


def test_batch_equals_single_runs_and_handles_edge_instances(gpu_ctx, ds):
    rng = np.random.default_rng(42)
    insts = [
        (np.zeros((0, 2)), 1.0, 3),                                   # empty
        (np.array([[1.0, 2.0, 3.0]]), 0.5, 1),                        # single point, core
        (rng.normal(0, 1, (500, 3)), 0.3, 5),
        (np.concatenate([c + rng.normal(0, 0.2, (400, 2))             # far apart: hash grid
                         for c in rng.uniform(-1e4, 1e4, (4, 2))]), 0.05, 4),
        (ds.blobs2d_100k(seed=1, scale=0.05).points, 0.5, 5),
        (np.zeros((0, 3)), 1.0, 3),                                   # empty 3D
        (ds.aniso3d_20m(seed=3, scale=0.0005).points, 0.05, 10),
    ]
    gpu_ctx.set_precision(1)
    labels, counts, _ = gpu_ctx.batch_dbscan(insts, with_stats=True)
    assert len(labels) == len(insts)
    for (pts, eps, mp), lab, k in zip(insts, labels, counts):
        if pts.shape[0] == 0:
            assert lab.shape == (0,) and k == 0
            continue
        single = gpu_ctx.dbscan(pts, eps, mp)
        assert np.array_equal(lab, single)
        assert k == (single.max() + 1 if (single >= 0).any() else 0)


def test_batch_rejects_bad_instance(gpu_ctx, gd):
    good = (np.zeros((4, 2)), 1.0, 2)
    for bad in [(np.zeros((4, 2)), 0.0, 2), (np.zeros((4, 2)), 1.0, 0),
                (np.array([[0.0, np.nan]]), 1.0, 1)]:
        with pytest.raises(gd.GdError) as e:
            gpu_ctx.batch_dbscan([good, bad])
        assert e.value.status == 1
    assert [l.tolist() for l in gpu_ctx.batch_dbscan([good])] == [[0, 0, 0, 0]]
