"""The oracle (CPU restatement) against the reference's own answers."""
import numpy as np
import pytest

from conftest import brute_dbscan, golden_cases


def test_ex_txt_known_answer(oracle):
    # test-datasets/ex.txt with common.h (EPS 1.5, MINPTS 3): three collinear trios
    ex = np.array([[1, 1], [2, 2], [3, 3], [10, 10], [11, 11], [12, 12],
                   [20, 20], [21, 21], [22, 22]], dtype=np.float64)
    lab, core, c = oracle.oracle_dbscan(ex, 1.5, 3)
    assert lab.tolist() == [0, 0, 0, 1, 1, 1, 2, 2, 2]
    assert core.tolist() == [False, True, False] * 3
    assert c["clusters"] == 3 and c["noise"] == 0 and c["border"] == 6


def test_oracle_matches_reference_golden(oracle):
    n = 0
    for name, pts, eps, mp, want in golden_cases():
        lab, _, _ = oracle.oracle_dbscan(pts, eps, mp)
        assert np.array_equal(lab, want), name
        n += 1
    assert n >= 50


def test_one_directional_pair_uses_sequential_relabel(oracle):
    X = [[1e-20, 0.0], [0.1, 0.0], [0.2, 0.0]]
    Y = [[-0.3, 0.0], [-0.4, 0.0], [-0.5, 0.0]]
    assert oracle.oracle_pred(np.array(X[0]), np.array(Y[0]), 0.3)
    assert not oracle.oracle_pred(np.array(Y[0]), np.array(X[0]), 0.3)
    lab, _, c = oracle.oracle_dbscan(np.array(X + Y), 0.3, 3)
    assert lab.tolist() == [0] * 6 and c["asym_pairs"] > 0 and c["sequential"] == 1
    lab, _, c = oracle.oracle_dbscan(np.array(Y + X), 0.3, 3)
    assert lab.tolist() == [0, 0, 0, 1, 1, 1]


@pytest.mark.parametrize("seed", range(6))
def test_oracle_3d_and_2d_vs_bruteforce(oracle, seed):
    rng = np.random.default_rng(100 + seed)
    for d in (2, 3):
        n = int(rng.integers(20, 300))
        pts = np.concatenate([rng.normal(0, 0.4, (n // 2, d)), rng.uniform(-2, 2, (n - n // 2, d))])
        if seed % 2:
            pts = np.round(pts * 4) / 4  # many exact ties on the eps boundary
        eps = float(rng.choice([0.25, 0.3, 0.5]))
        mp = int(rng.integers(1, 10))
        lab, _, _ = oracle.oracle_dbscan(pts, eps, mp)
        assert np.array_equal(lab, brute_dbscan(pts, eps, mp)), (d, n, eps, mp)


def test_oracle_rejects_bad_input(oracle):
    with pytest.raises(ValueError):
        oracle.oracle_dbscan(np.array([[0.0, np.nan]]), 1.0, 1)
    with pytest.raises(ValueError):
        oracle.oracle_dbscan(np.zeros((3, 2)), 0.0, 1)
    with pytest.raises(ValueError):
        oracle.oracle_dbscan(np.zeros((3, 2)), 1.0, 0)


def test_oracle_vs_live_reference(oracle):
    """When the reference checkout is present, compare on fresh random inputs."""
    if not oracle.ref_available():
        pytest.skip("reference checkout not present")
    rng = np.random.default_rng(777)
    for _ in range(40):
        n = int(rng.integers(10, 3000))
        pts = rng.normal(0, 1, (n, 2)) * 10 ** rng.uniform(-2, 2)
        eps = float(np.std(pts) * rng.uniform(0.02, 0.3))
        mp = int(rng.integers(1, 16))
        lab, _, _ = oracle.oracle_dbscan(pts, eps, mp)
        ref, _ = oracle.ref_rtree_dbscan(pts, eps, mp)
        assert np.array_equal(lab, ref)


def test_reference_multicore_baseline_runs(oracle):
    """The reference's multicore CPU DBSCAN (a timed baseline only: it counts
    neighbours without the point itself and tests float32 sqrt(d2) <= eps, so
    its clusters are not compared with the exact ones) builds from the checkout
    and gives the same cluster count on repeated runs and thread counts."""
    from oracle import build as obuild
    if obuild.build_ref_multicore() is None:
        pytest.skip("reference checkout not present")
    rng = np.random.default_rng(5)
    pts = np.concatenate([rng.normal(c, 0.3, (400, 2)) for c in ((0, 0), (5, 5), (0, 5))])
    k1 = oracle.ref_multicore_dbscan(pts, 0.3, 5, threads=1)
    k4 = oracle.ref_multicore_dbscan(pts, 0.3, 5, threads=4)
    assert k1 == k4 >= 3


@pytest.mark.parametrize("spacing,offset", [(0.1, 0.0), (0.3, 1000.0), (0.001, 12.3)])
def test_quantised_inputs_stay_below_the_one_directional_pair_cap(oracle, spacing, offset):
    # A pair is a neighbour one way only when the query box and the distance test
    # disagree in the last bit (the case above: a coordinate near 0 beside one at
    # eps).  Lattices with spacing equal to eps, and data rounded to a decimal
    # step, produce none, far from the 2,048 pairs the device's merge replay holds.
    xs = np.arange(100) * spacing + offset
    g = np.stack(np.meshgrid(xs, xs, indexing="ij"), -1).reshape(-1, 2)
    _, _, c = oracle.oracle_dbscan(g, spacing, 4)
    assert c["asym_pairs"] == 0
    rng = np.random.default_rng(7)
    dec = int(round(-np.log10(spacing)))
    r = np.round(rng.uniform(0, 500 * spacing, size=(20000, 2)), dec) + offset
    _, _, c = oracle.oracle_dbscan(r, spacing, 4)
    assert c["asym_pairs"] == 0
