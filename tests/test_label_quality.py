"""Label-quality report (gd_label_quality_compare, gbdbscan_check) against the
reference's own cluster check (test-results/cluster-check.cpp:41-199).

The bar is bit-exact: the per-point Jaccard scores are the same double
divisions of the same integers, summed in point order, so the report's two
ratios must equal the reference's doubles exactly (its harness prints them
with every bit).  The golden pairs (tests/golden/make_label_quality.py) run
everywhere; the comparison against the reference program itself runs where the
reference checkout can be compiled.  Host code only: no GPU."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "label_quality_golden.npz")
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def _golden():
    z = np.load(GOLDEN)
    for name in sorted({k.split("/")[0] for k in z.files}):
        yield name, z[f"{name}/a"], z[f"{name}/b"], {
            k: z[f"{name}/{k}"].item()
            for k in ("score", "mismatch_loss", "noise_mismatch", "noise_agree", "max1", "max2")}


def _check(got, want):
    assert got["score"] == want["score"]
    assert got["mismatch_loss"] == want["mismatch_loss"]
    assert got["noise_mismatch"] == want["noise_mismatch"]
    assert got["noise_agree"] == want["noise_agree"]


def test_golden_pairs(built_lib, gd):
    n = 0
    for name, a, b, want in _golden():
        got = gd.label_quality(a, b, noise=0)
        _check(got, want)
        assert got["n"] == a.shape[0], name
        n += 1
    assert n >= 9


def test_library_noise_convention(built_lib, gd):
    """The same pair in this library's convention (noise -2, clusters 0..K-1)
    gives the same report."""
    for name, a, b, want in _golden():
        got = gd.label_quality(np.where(a == 0, -2, a - 1), np.where(b == 0, -2, b - 1))
        _check(got, want)


def test_edge_cases_and_errors(built_lib, gd):
    got = gd.label_quality(np.zeros(0, np.int32), np.zeros(0, np.int32))
    assert got["score"] == 1.0 and got["n"] == 0
    got = gd.label_quality([5], [7])
    assert got["score"] == 1.0 and got["clusters_a"] == 1
    got = gd.label_quality([-2, 3], [3, -2])
    assert got["score"] == 0.0 and got["noise_mismatch"] == 2
    # arbitrary cluster ids (negative, large) are just ids
    got = gd.label_quality([-7, -7, 2 ** 31 - 1], [4, 4, 9], noise=0)
    assert got["score"] == 1.0 and got["clusters_a"] == 2
    with pytest.raises(ValueError):
        gd.label_quality([1, 2], [1])
    lib = gd.load_library()
    assert lib.gd_label_quality_compare(None, None, 3, 0, gd.api.GdLabelQuality()) == 1  # EINVAL
    assert lib.gd_label_quality_compare(None, None, 0, 0, None) == 1


def _ref_exe():
    from oracle import build as ob
    try:
        return ob.build_ref_check()
    except Exception:
        return None


def test_against_reference_program(built_lib, gd):
    exe = _ref_exe()
    if exe is None:
        pytest.skip("reference checkout absent")
    import make_label_quality as mk
    rng = np.random.default_rng(9)
    for t in range(40):
        n = int(rng.integers(1, 3000))
        k = int(rng.integers(1, 80))
        a = rng.integers(0, k + 1, n)
        mode = t % 4
        if mode == 0:
            b = a.copy()
        elif mode == 1:
            b = np.where(rng.random(n) < 0.1, rng.integers(0, k + 1, n), a)
        elif mode == 2:
            b = (a * 3 + rng.integers(0, 2, n)) % (k + 3)
        else:
            b = rng.integers(0, int(rng.integers(1, 10)) + 1, n)
        want = mk.run_reference(exe, a.astype(np.int32), b.astype(np.int32))
        _check(gd.label_quality(a, b, noise=0), want)


def test_cli_matches_reference_lines(built_lib, tmp_path):
    exe = os.path.join(os.path.dirname(built_lib), "gbdbscan_check")
    for name, a, b, want in list(_golden())[:4]:
        fa, fb = tmp_path / f"{name}_a.txt", tmp_path / f"{name}_b.txt"
        np.savetxt(fa, a, fmt="%d")
        np.savetxt(fb, b, fmt="%d")
        out = subprocess.run([exe, str(fa), str(fb)], capture_output=True, text=True,
                             check=True).stdout
        assert f"Final Error metric: {want['score']:f}" in out, out
        assert f"fraction lost due to mismatches between clusters: {want['mismatch_loss']:f}" in out
        assert (f"mismatched noise points: {want['noise_mismatch']}, "
                f"agreement noise points: {want['noise_agree']}") in out
        assert f"num clusters in list1, list2: {want['max1']},{want['max2']}" in out
