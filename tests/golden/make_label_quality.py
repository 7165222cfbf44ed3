"""Generate golden fixtures for the label-quality report from the reference's own
cluster check.

Runs the reference's test-results/cluster-check.cpp (compiled from the
reference checkout by oracle/build.py into oracle/_ref/ref_cluster_check, its
two ratios printed with every bit) on seeded label pairs, and stores the pairs
with the reference's results in label_quality_golden.npz.  Labels use the
reference's convention: 0 = noise, clusters 1..K.

    python tests/golden/make_label_quality.py      (needs the reference checkout)

Cases (label_pairs()):
  same_perm     one labelling against itself with its cluster ids permuted
  split_merge   clusters split in two and neighbouring clusters merged
  noise_flip    a share of points moved to or from noise
  all_noise     every point noise in both
  one_vs_many   one cluster against a fine partition of the same points
  random_*      seeded random labellings with noise, of mixed cluster sizes
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "label_quality_golden.npz")


def label_pairs():
    """(name, a, b) label pairs, 0 = noise."""
    rng = np.random.default_rng(42)
    out = []
    a = rng.integers(0, 12, 1500)
    perm = np.concatenate([[0], rng.permutation(np.arange(1, 12))])
    out.append(("same_perm", a, perm[a]))
    a = rng.integers(1, 9, 1200)
    b = a * 2 - (rng.random(a.shape) < 0.4)                    # each cluster split in two
    b = np.where(np.isin(a, [3, 4]), 100, b)                   # clusters 3 and 4 merged
    out.append(("split_merge", a, b))
    a = rng.integers(0, 7, 1000)
    b = a.copy()
    flip = rng.random(a.shape) < 0.15
    b[flip] = np.where(b[flip] == 0, rng.integers(1, 7, int(flip.sum())), 0)
    out.append(("noise_flip", a, b))
    out.append(("all_noise", np.zeros(300, np.int64), np.zeros(300, np.int64)))
    a = np.ones(800, np.int64)
    out.append(("one_vs_many", a, rng.integers(1, 40, 800)))
    for s in range(4):
        r = np.random.default_rng(100 + s)
        n = int(r.integers(50, 2500))
        k = int(r.integers(1, 60))
        sizes = r.zipf(1.6, k).astype(np.float64)
        p = np.concatenate([[r.uniform(0.02, 0.4)], sizes / sizes.sum() * 0.8])
        p /= p.sum()
        a = r.choice(k + 1, size=n, p=p)
        b = np.where(r.random(n) < 0.8, a, r.choice(k + 1, size=n, p=p))
        out.append((f"random_{s}", a, b))
    return [(name, np.asarray(a, np.int32), np.asarray(b, np.int32)) for name, a, b in out]


_LINE = {
    "noise": re.compile(r"mismatched noise points: (-?\d+), agreement noise points: (-?\d+)"),
    "lost": re.compile(r"fraction lost due to mismatches between clusters: (\S+)"),
    "final": re.compile(r"Final Error metric: (\S+)"),
    "clusters": re.compile(r"num clusters in list1, list2: (-?\d+),(-?\d+)"),
}


def run_reference(exe: str, a: np.ndarray, b: np.ndarray) -> dict:
    """The reference cluster check's report on one pair (0 = noise)."""
    with tempfile.TemporaryDirectory() as d:
        fa, fb = os.path.join(d, "a.txt"), os.path.join(d, "b.txt")
        np.savetxt(fa, a, fmt="%d")
        np.savetxt(fb, b, fmt="%d")
        text = subprocess.run([exe, fa, fb], capture_output=True, text=True, check=True).stdout
    m = {k: r.search(text) for k, r in _LINE.items()}
    assert all(m.values()), text
    return {"noise_mismatch": int(m["noise"].group(1)), "noise_agree": int(m["noise"].group(2)),
            "mismatch_loss": float(m["lost"].group(1)), "score": float(m["final"].group(1)),
            "max1": int(m["clusters"].group(1)), "max2": int(m["clusters"].group(2))}


def main():
    sys.path.insert(0, ROOT)
    from oracle import build as ob
    exe = ob.build_ref_check()
    if exe is None:
        raise SystemExit("the reference checkout is absent: nothing to generate")
    z = {}
    for name, a, b in label_pairs():
        r = run_reference(exe, a, b)
        z[f"{name}/a"] = a
        z[f"{name}/b"] = b
        for k, v in r.items():
            z[f"{name}/{k}"] = np.array(v)
    np.savez_compressed(OUT, **z)
    print(OUT, len(z))


if __name__ == "__main__":
    main()
