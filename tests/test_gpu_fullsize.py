"""Full-size parity: the 10,000,000-point 2D set and the 20,000,000-point 3D set
with planted eps(1 +/- 1e-7) pairs, bit-exact against the oracle (run on all
host cores), in both precision modes, plus size-independent properties (core
flags agree with a recount on a random sample, labels identical across
precisions and repeated runs)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check_sample_core(points, eps, minpts, core, rng, m=2000):
    """Recount |N(p)| for a random sample by brute force (same float64 predicate
    as the oracle, box test included) and compare with the returned core flags."""
    n, d = points.shape
    idx = rng.choice(n, size=min(m, n), replace=False)
    e2 = eps * eps
    for i in idx:
        p = points[i]
        lo, hi = p - eps, p + eps
        box = np.all((points >= lo) & (points <= hi), axis=1)
        q = points[box]
        diff = p - q
        d2 = diff[:, 0] * diff[:, 0] + diff[:, 1] * diff[:, 1]
        if d == 3:
            d2 = d2 + diff[:, 2] * diff[:, 2]
        assert bool(core[i]) == (int(np.count_nonzero(d2 <= e2)) >= minpts)


@pytest.mark.parametrize("maker", ["zipf2d_10m", "aniso3d_20m"])
def test_full_size_vs_oracle(gpu_ctx, ds, oracle, maker):
    inst = getattr(ds, maker)(seed=0)
    olab, ocore, _ = oracle.oracle_dbscan(inst.points, inst.eps, inst.minpts,
                                          nthreads=os.cpu_count() or 1)
    for prec in (0, 1):
        gpu_ctx.set_precision(prec)
        lab, core = gpu_ctx.dbscan(inst.points, inst.eps, inst.minpts, with_core=True)
        assert np.array_equal(core.astype(bool), ocore.astype(bool)), prec
        assert np.array_equal(lab, olab), prec
        st = gpu_ctx.stats()
        assert st["n_points"] == inst.n
        if prec == 1 and maker == "aniso3d_20m":
            assert st["precision_used"] == 1 and st["band_retests"] > 0
    again = gpu_ctx.dbscan(inst.points, inst.eps, inst.minpts)
    assert np.array_equal(again, olab)
    _check_sample_core(inst.points, inst.eps, inst.minpts, ocore, np.random.default_rng(7),
                       m=40)
