"""Synthetic workload generators: seeded, shaped as specified."""
import numpy as np


def test_blobs2d_shape_and_determinism(ds):
    a = ds.blobs2d_100k(seed=0)
    b = ds.blobs2d_100k(seed=0)
    assert a.points.shape == (100_000, 2) and a.eps == 0.5 and a.minpts == 5
    assert np.array_equal(a.points, b.points)
    assert not np.array_equal(a.points, ds.blobs2d_100k(seed=1).points)


def test_zipf2d_scaled(ds):
    inst = ds.zipf2d_10m(scale=0.01)
    assert inst.points.shape == (100_000, 2) and inst.eps == 0.3 and inst.minpts == 8


def test_aniso3d_scaled_has_planted_pairs(ds):
    inst = ds.aniso3d_20m(scale=0.005)
    assert inst.points.shape == (100_000, 3) and inst.eps == 0.05 and inst.minpts == 10
    assert inst.meta["planted_pairs"] == 500


def test_batch_instances(ds):
    insts = ds.batch4096(count=8, scale=0.01)
    assert len(insts) == 8
    for inst in insts:
        assert inst.dim in (2, 3) and 4 <= inst.minpts <= 32 and inst.eps > 0


def test_tiny_cases(ds):
    names = [c.name for c in ds.tiny_cases()]
    assert "ex_txt" in names and "eps_exact_345" in names
