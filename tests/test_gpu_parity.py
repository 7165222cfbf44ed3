"""GPU parity: labels from libgbdbscan.so (through the C ABI) against the oracle
and the reference's golden labels.  The bar is bit-exact: identical labels,
identical core flags (NOISE=-2, clusters 0..K-1 by smallest core index)."""
import numpy as np
import pytest

from conftest import brute_dbscan, golden_cases

pytestmark = pytest.mark.gpu

PRECISIONS = [0, 1]  # GD_PREC_FP64, GD_PREC_FP32_BAND


def run(ctx, pts, eps, mp, prec, with_core=True):
    ctx.set_precision(prec)
    return ctx.dbscan(pts, eps, mp, with_core=with_core)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_golden_reference_labels(gpu_ctx, prec):
    n = 0
    for name, pts, eps, mp, want in golden_cases():
        lab, _ = run(gpu_ctx, pts, eps, mp, prec)
        assert np.array_equal(lab, want), name
        n += 1
    assert n >= 50


@pytest.mark.parametrize("prec", PRECISIONS)
def test_tiny_cases_vs_oracle(gpu_ctx, ds, oracle, prec):
    for inst in ds.tiny_cases():
        lab, core = run(gpu_ctx, inst.points, inst.eps, inst.minpts, prec)
        olab, ocore, _ = oracle.oracle_dbscan(inst.points, inst.eps, inst.minpts)
        assert np.array_equal(lab, olab), inst.name
        assert np.array_equal(core, ocore), inst.name


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("seed", range(8))
def test_random_small_vs_bruteforce(gpu_ctx, prec, seed):
    rng = np.random.default_rng(1000 + seed)
    for d in (2, 3):
        n = int(rng.integers(2, 400))
        pts = np.concatenate([rng.normal(0, 0.4, (n // 2, d)), rng.uniform(-2, 2, (n - n // 2, d))])
        if seed % 2:
            pts = np.round(pts * 4) / 4
        eps = float(rng.choice([0.25, 0.3, 0.5, 1.0]))
        mp = int(rng.integers(1, 40))
        lab, _ = run(gpu_ctx, pts, eps, mp, prec)
        assert np.array_equal(lab, brute_dbscan(pts, eps, mp)), (d, n, eps, mp)


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("seed", range(4))
def test_random_medium_vs_oracle(gpu_ctx, oracle, prec, seed):
    rng = np.random.default_rng(2000 + seed)
    for d in (2, 3):
        n = int(rng.integers(1000, 60000))
        k = int(rng.integers(1, 30))
        centres = rng.uniform(0, 50, (k, d))
        pts = np.concatenate([centres[rng.integers(0, k, n)] + rng.normal(0, rng.uniform(0.2, 3), (n, d)),
                              rng.uniform(0, 50, (n // 10, d))])
        pts = pts * 10 ** rng.uniform(-3, 3) + rng.uniform(-1e3, 1e3)
        eps = float(np.std(pts) * rng.uniform(0.005, 0.05))
        mp = int(rng.integers(2, 40))
        lab, core = run(gpu_ctx, pts, eps, mp, prec)
        olab, ocore, _ = oracle.oracle_dbscan(pts, eps, mp)
        assert np.array_equal(core, ocore)
        assert np.array_equal(lab, olab)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_blobs2d_100k_golden(gpu_ctx, prec):
    (name, pts, eps, mp, want), = list(golden_cases({"c1_seed0"}))
    lab, _ = run(gpu_ctx, pts, eps, mp, prec)
    assert np.array_equal(lab, want)


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("maker,scale", [("zipf2d_10m", 0.02), ("aniso3d_20m", 0.01)])
def test_scaled_workloads_vs_oracle(gpu_ctx, ds, oracle, prec, maker, scale):
    inst = getattr(ds, maker)(seed=0, scale=scale)
    lab, core = run(gpu_ctx, inst.points, inst.eps, inst.minpts, prec)
    olab, ocore, _ = oracle.oracle_dbscan(inst.points, inst.eps, inst.minpts)
    assert np.array_equal(core, ocore)
    assert np.array_equal(lab, olab)
    st = gpu_ctx.stats()
    if prec == 1:
        assert st["precision_used"] == 1 and st["tests_fp32"] > 0
        if maker == "aniso3d_20m":
            assert st["band_retests"] > 0   # planted eps*(1 +/- 1e-7) pairs


def test_staged_api_equals_fused_and_minpts_rerun(gpu_ctx, ds, oracle):
    inst = ds.zipf2d_10m(seed=1, scale=0.005)
    gpu_ctx.set_precision(0)
    lab_f, st = gpu_ctx.dbscan_fused(inst.points, inst.eps, inst.minpts)
    gpu_ctx.index_build(inst.points, inst.eps)
    for mp in (inst.minpts, 3, 20):
        gpu_ctx.expand(mp)
        lab = gpu_ctx.get_result()
        olab, _, c = oracle.oracle_dbscan(inst.points, inst.eps, mp)
        assert np.array_equal(lab, olab), mp
        if mp == inst.minpts:
            assert np.array_equal(lab, lab_f)
            assert st["n_clusters"] == c["clusters"] and st["n_noise"] == c["noise"]


def test_device_resident_input(gpu_ctx, ds, oracle):
    import torch
    inst = ds.aniso3d_20m(seed=2, scale=0.005)
    t = torch.from_numpy(inst.points).cuda()
    gpu_ctx.set_precision(1)
    lab, core = gpu_ctx.dbscan(t, inst.eps, inst.minpts, with_core=True)
    assert lab.is_cuda
    olab, ocore, _ = oracle.oracle_dbscan(inst.points, inst.eps, inst.minpts)
    assert np.array_equal(lab.cpu().numpy(), olab)
    assert np.array_equal(core.cpu().numpy().astype(bool), ocore)


def test_deterministic_repeat(gpu_ctx, ds):
    inst = ds.zipf2d_10m(seed=3, scale=0.01)
    a, _ = run(gpu_ctx, inst.points, inst.eps, inst.minpts, 1)
    b, _ = run(gpu_ctx, inst.points, inst.eps, inst.minpts, 1)
    c, _ = run(gpu_ctx, inst.points, inst.eps, inst.minpts, 0)
    assert np.array_equal(a, b) and np.array_equal(a, c)


def test_errors_are_status_codes(gpu_ctx, gd):
    pts = np.zeros((4, 2))
    for bad in (lambda: gpu_ctx.dbscan(np.array([[0.0, np.nan], [1.0, 1.0]]), 1.0, 2),
                lambda: gpu_ctx.dbscan(pts, 0.0, 2),
                lambda: gpu_ctx.dbscan(pts, float("inf"), 2),
                lambda: gpu_ctx.dbscan(pts, 1.0, 0),
                lambda: gpu_ctx.dbscan(np.zeros((4, 4)), 1.0, 2)):
        with pytest.raises(gd.GdError) as e:
            bad()
        assert e.value.status == 1
    # a grid far beyond the cell-table limit is refused, not attempted
    with pytest.raises(gd.GdError) as e:
        gpu_ctx.dbscan(np.array([[0.0, 0.0], [1e9, 1e9]]), 1e-3, 1)
    assert e.value.status == 4
    # the context stays usable after errors
    lab = gpu_ctx.dbscan(np.array([[0.0, 0.0], [0.1, 0.0], [5.0, 5.0]]), 0.5, 2)
    assert lab.tolist() == [0, 0, -2]


def test_empty_and_single(gpu_ctx):
    assert gpu_ctx.dbscan(np.zeros((0, 2)), 1.0, 1).shape == (0,)
    assert gpu_ctx.dbscan(np.array([[1.0, 2.0, 3.0]]), 1.0, 1).tolist() == [0]
    assert gpu_ctx.dbscan(np.array([[1.0, 2.0, 3.0]]), 1.0, 2).tolist() == [-2]


def test_cli_end_to_end(built_lib, tmp_path, ds, oracle):
    import os
    import subprocess
    inst = ds.blobs2d_100k(seed=4, scale=0.05)
    csv = tmp_path / "pts.csv"
    ds.write_csv(str(csv), inst.points)
    out = tmp_path / "labels.txt"
    exe = os.path.join(os.path.dirname(built_lib), "gbdbscan_main")
    r = subprocess.run([exe, str(csv), "--eps", str(inst.eps), "--minpts", str(inst.minpts),
                        "--out", str(out)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    olab, _, c = oracle.oracle_dbscan(inst.points, inst.eps, inst.minpts)
    assert f"Final cluster after merging: {c['clusters']}" in r.stdout
    assert f"Number of noises: {c['noise']}" in r.stdout
    assert np.array_equal(np.loadtxt(str(out), dtype=np.int32), olab)


@pytest.mark.parametrize("dim", [2, 3])
def test_cli_binary_f64_input(built_lib, tmp_path, ds, oracle, dim):
    """The CLI's binary input (raw row-major float64, '.f64'), the fast path
    that replaces the text parse of ImportDataset (main.cu:469-498): same
    labels as the oracle and the same report lines as the CSV path."""
    import os
    import subprocess
    inst = ds.blobs2d_100k(seed=8, scale=0.05) if dim == 2 else ds.aniso3d_20m(seed=8,
                                                                                scale=0.0005)
    raw = tmp_path / "pts.f64"
    np.ascontiguousarray(inst.points, dtype=np.float64).tofile(str(raw))
    out = tmp_path / "labels.txt"
    exe = os.path.join(os.path.dirname(built_lib), "gbdbscan_main")
    r = subprocess.run([exe, str(raw), "--eps", str(inst.eps), "--minpts", str(inst.minpts),
                        "--dim", str(dim), "--out", str(out)], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0, r.stderr
    olab, _, c = oracle.oracle_dbscan(inst.points, inst.eps, inst.minpts)
    assert f"Final cluster after merging: {c['clusters']}" in r.stdout
    assert f"Number of noises: {c['noise']}" in r.stdout
    assert np.array_equal(np.loadtxt(str(out), dtype=np.int32), olab)


@pytest.mark.parametrize("prec", PRECISIONS)
@pytest.mark.parametrize("d,extent,hashed", [(2, 1e4, False), (2, 1e7, True),
                                             (3, 1e2, False), (3, 1e4, True)])
def test_sparse_grid_vs_oracle(gpu_ctx, oracle, prec, d, extent, hashed):
    """Far-apart blobs: the eps-cell grid exceeds the dense cell table.  Rows
    are then looked up through a table of rows when there are few enough of
    them, else through the hash of occupied rows (64-bit keys)."""
    rng = np.random.default_rng(31 + d)
    centres = rng.uniform(-extent, extent, (6, d))
    pts = np.concatenate([c + rng.normal(0, 0.2, (3000, d)) for c in centres] +
                         [rng.uniform(-extent, extent, (500, d))])
    pts = pts[rng.permutation(len(pts))]
    lab, core = run(gpu_ctx, pts, 0.05, 6, prec)
    st = gpu_ctx.stats()
    assert st["key_bits"] > 26                      # beyond the dense cell table
    if hashed:
        assert st["grid_cells"] == 0                # no occupancy table: the hash
    else:
        assert 1 < st["grid_cells"] < 2 ** 27       # one occupancy bit per row (+1)
    olab, ocore, _ = oracle.oracle_dbscan(pts, 0.05, 6)
    assert np.array_equal(core, ocore)
    assert np.array_equal(lab, olab)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_far_from_origin_disables_shortcuts(gpu_ctx, oracle, prec):
    """|x| far above eps * 2^30: no box-test shortcut, no float32 filter, no cell
    classification -- every decision is the plain float64 predicate."""
    rng = np.random.default_rng(77)
    pts = 3e9 + np.concatenate([rng.normal(0, 1.0, (3000, 2)), rng.uniform(-20, 20, (500, 2))])
    lab, core = run(gpu_ctx, pts, 0.25, 5, prec)
    assert gpu_ctx.stats()["precision_used"] == 0
    olab, ocore, _ = oracle.oracle_dbscan(pts, 0.25, 5)
    assert np.array_equal(core, ocore)
    assert np.array_equal(lab, olab)


@pytest.mark.parametrize("prec", PRECISIONS)
def test_points_on_cell_boundaries_vs_oracle(gpu_ctx, oracle, prec):
    """Coordinates on, and a few ulps either side of, the grid's cell boundaries
    lo + c f (lo = 0, f the default cell side eps * 0.5 (1 + 2^-16)): the cell
    keys' float32 path must hand these to the float64 formula.  The lattice
    also puts many pairs at 2f = eps (1 + 2^-16), just beyond eps, and the ulp
    offsets move some of them across.  Labels and core flags must stay the
    oracle's."""
    rng = np.random.default_rng(77)
    for d, cells, n, mp in ((2, 200, 60000, 12), (3, 40, 60000, 26)):
        eps = 0.3 if d == 2 else 0.05
        f = eps * (0.5 * (1 + 2.0 ** -16))
        c = rng.integers(0, cells, (n, d)).astype(np.float64)
        base = c * f
        ulps = rng.integers(-3, 4, (n, d)).astype(np.float64)
        pts = np.maximum(base + ulps * np.spacing(np.maximum(base, f)), 0.0)
        pts[0] = 0.0
        lab, core = run(gpu_ctx, pts, eps, mp, prec)
        olab, ocore, _ = oracle.oracle_dbscan(pts, eps, mp)
        assert np.array_equal(core, ocore), d
        assert np.array_equal(lab, olab), d
        assert 0 < int(ocore.sum()) < n and olab.max() >= 1, d   # a real mix of outcomes
