"""Seeded synthetic point sets standing in for the reference's datasets.

The reference (CUDA-DClust+) was measured on external 2D/3D datasets that are
not available here; its input format is a headerless CSV with one point per line
and DIMENSION comma-separated doubles (main.cu:469-498).  These generators make
point sets with the shapes, sizes and value distributions of the five workloads
this project is measured on, from a numpy PCG64 generator with a recorded seed:

  blobs2d_100k      2D, 100,000 points: 20 isotropic Gaussians x 4,500 (centres
                    U[0,100]^2, sigma U[0.5,2.0]) + 10,000 U[0,100]^2 noise;
                    eps=0.5, minpts=5.
  zipf2d_10m        2D, 10,000,000 points: 500 Gaussians (centres U[0,1000]^2,
                    sigma log-U[0.5,5], sizes Zipf s=1.1 normalised to 9.5M) +
                    500,000 U[0,1000]^2 noise; eps=0.3, minpts=8.
  aniso3d_20m       3D, 20,000,000 points: 64 rotated anisotropic Gaussians
                    (axis sigmas U[0.02,0.5], centres U[0,10]^3) + 10% U[0,10]^3
                    noise + 1% planted pairs at distance eps*(1 +/- 1e-7);
                    eps=0.05, minpts=10.
  batch4096         4,096 instances, n log-U[256, 200,000], d in {2,3} 50/50,
                    1-32 blobs, 5-20% noise, eps = median exact 4th-NN distance
                    (over a sample of query points), minpts U[4,32].
  serve stream      Poisson arrivals, sizes log-U[1,000, 2,000,000], per-request
                    eps/minpts as for batch4096.

All point arrays are float64, C-contiguous, shape (n, d) -- the same
array-of-structures layout the reference keeps in host and device memory.
Every generator takes a ``scale`` in (0, 1] that shrinks the point counts while
keeping the densities of the blobs (so small test cases look like the big ones).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Instance:
    points: np.ndarray          # (n, d) float64
    eps: float
    minpts: int
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.points.shape[0])

    @property
    def dim(self) -> int:
        return int(self.points.shape[1])


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.PCG64(seed))


def _finish(rng: np.random.Generator, parts, shuffle=True) -> np.ndarray:
    pts = np.concatenate(parts, axis=0)
    if shuffle:
        pts = pts[rng.permutation(pts.shape[0])]
    return np.ascontiguousarray(pts, dtype=np.float64)


def blobs2d_100k(seed: int = 0, scale: float = 1.0) -> Instance:
    """2D, 20 isotropic Gaussian blobs of 4,500 points + 10,000 uniform noise."""
    rng = _rng(seed)
    nb = max(1, int(round(4500 * scale)))
    nn = int(round(10000 * scale))
    centres = rng.uniform(0.0, 100.0, size=(20, 2))
    sigmas = rng.uniform(0.5, 2.0, size=20)
    parts = [centres[i] + sigmas[i] * rng.standard_normal((nb, 2)) for i in range(20)]
    parts.append(rng.uniform(0.0, 100.0, size=(nn, 2)))
    return Instance(_finish(rng, parts), 0.5, 5, "blobs2d_100k",
                    {"seed": seed, "scale": scale})


def zipf2d_10m(seed: int = 0, scale: float = 1.0) -> Instance:
    """2D, 500 Zipf-sized Gaussian blobs (9.5M points) + 500K uniform noise.

    With scale < 1 the blob sizes and the noise count shrink and the domain
    shrinks by sqrt(scale), so densities (and hence neighbour counts per point)
    stay those of the full-size set.
    """
    rng = _rng(seed)
    total_blob = int(round(9_500_000 * scale))
    n_noise = int(round(500_000 * scale))
    side = 1000.0 * math.sqrt(scale)
    k = np.arange(1, 501, dtype=np.float64)
    w = k ** -1.1
    w /= w.sum()
    sizes = np.floor(w * total_blob).astype(np.int64)
    sizes[: total_blob - int(sizes.sum())] += 1
    centres = rng.uniform(0.0, side, size=(500, 2))
    sigmas = np.exp(rng.uniform(math.log(0.5), math.log(5.0), size=500))
    parts = []
    for i in range(500):
        if sizes[i] > 0:
            parts.append(centres[i] + sigmas[i] * rng.standard_normal((int(sizes[i]), 2)))
    parts.append(rng.uniform(0.0, side, size=(n_noise, 2)))
    return Instance(_finish(rng, parts), 0.3, 8, "zipf2d_10m",
                    {"seed": seed, "scale": scale, "noise_domain": [0.0, side]})


def _random_rotation(rng: np.random.Generator) -> np.ndarray:
    q, r = np.linalg.qr(rng.standard_normal((3, 3)))
    q *= np.sign(np.diag(r))
    return q


def aniso3d_20m(seed: int = 0, scale: float = 1.0) -> Instance:
    """3D, 64 rotated anisotropic Gaussians + 10% noise + 1% planted eps-pairs.

    The planted pairs (half at eps*(1-1e-7), half at eps*(1+1e-7), random
    directions) sit so close to the eps boundary that a float32 distance cannot
    decide them; they exercise the float64 re-test band.  Half of the pair
    anchors are existing blob points, half are uniform in the domain.
    """
    rng = _rng(seed)
    eps = 0.05
    n_total = int(round(20_000_000 * scale))
    n_noise = int(round(0.10 * n_total))
    n_pair_pts = 2 * (int(round(0.01 * n_total)) // 2)
    n_blob = n_total - n_noise - n_pair_pts
    side = 10.0 * scale ** (1.0 / 3.0)
    sizes = np.full(64, n_blob // 64, dtype=np.int64)
    sizes[: n_blob - int(sizes.sum())] += 1
    centres = rng.uniform(0.0, side, size=(64, 3))
    parts = []
    for i in range(64):
        # axis sigmas shrink with the domain, so a scaled-down set keeps the
        # blob densities (and neighbour counts) of the full-size one
        sig = rng.uniform(0.02, 0.5, size=3) * scale ** (1.0 / 3.0)
        rot = _random_rotation(rng)
        z = rng.standard_normal((int(sizes[i]), 3)) * sig
        parts.append(centres[i] + z @ rot.T)
    blobs = np.concatenate(parts, axis=0)
    noise = rng.uniform(0.0, side, size=(n_noise, 3))
    npairs = n_pair_pts // 2
    n_anchor_blob = npairs // 2
    anchors = np.concatenate([
        blobs[rng.integers(0, max(1, blobs.shape[0]), size=n_anchor_blob)] if blobs.shape[0] else
        rng.uniform(0.0, side, size=(n_anchor_blob, 3)),
        rng.uniform(0.0, side, size=(npairs - n_anchor_blob, 3)),
    ], axis=0)
    # jitter the anchors off the existing points so the pair is a fresh pair
    anchors = anchors + rng.uniform(-eps, eps, size=anchors.shape)
    dirs = rng.standard_normal((npairs, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    factor = np.where(np.arange(npairs) % 2 == 0, 1.0 - 1e-7, 1.0 + 1e-7)
    partners = anchors + (eps * factor)[:, None] * dirs
    return Instance(_finish(rng, [blobs, noise, anchors, partners]), eps, 10, "aniso3d_20m",
                    {"seed": seed, "scale": scale, "planted_pairs": int(npairs)})


def median_knn_eps(points: np.ndarray, k: int = 4, max_queries: int = 2048,
                   seed: int = 0) -> float:
    """Median exact k-th nearest-neighbour distance (self excluded).

    The distances are exact (scipy cKDTree); the median is taken over at most
    ``max_queries`` query points drawn without replacement.
    """
    from scipy.spatial import cKDTree
    n = points.shape[0]
    if n <= k:
        return 1.0
    tree = cKDTree(points)
    rng = _rng(seed)
    q = points if n <= max_queries else points[rng.choice(n, size=max_queries, replace=False)]
    d, _ = tree.query(q, k=k + 1)
    return float(np.median(d[:, k]))


def mixture_instance(rng: np.random.Generator, n: int, dim: int,
                     with_eps: bool = True) -> Instance:
    """One instance of the batched / served workloads (1-32 blobs, 5-20% noise)."""
    nblobs = int(rng.integers(1, 33))
    noise_frac = float(rng.uniform(0.05, 0.20))
    n_noise = int(round(noise_frac * n))
    n_blob = n - n_noise
    side = 100.0
    centres = rng.uniform(0.0, side, size=(nblobs, dim))
    sig = np.exp(rng.uniform(math.log(0.5), math.log(5.0), size=nblobs))
    w = rng.dirichlet(np.ones(nblobs))
    sizes = np.floor(w * n_blob).astype(np.int64)
    sizes[: n_blob - int(sizes.sum())] += 1
    parts = [centres[i] + sig[i] * rng.standard_normal((int(sizes[i]), dim))
             for i in range(nblobs) if sizes[i] > 0]
    parts.append(rng.uniform(0.0, side, size=(n_noise, dim)))
    pts = _finish(rng, parts)
    minpts = int(rng.integers(4, 33))
    eps = median_knn_eps(pts, 4, seed=int(rng.integers(0, 2**31))) if with_eps else 1.0
    return Instance(pts, eps, minpts, f"mix{dim}d_{n}",
                    {"nblobs": nblobs, "noise_frac": noise_frac})


def batch_sizes(rng: np.random.Generator, count: int, lo: int, hi: int) -> np.ndarray:
    return np.exp(rng.uniform(math.log(lo), math.log(hi), size=count)).astype(np.int64)


def _batch_one(args) -> Instance:
    seed, i, n, dim = args
    inst = mixture_instance(_rng(seed * 1_000_003 + i + 1), n, dim)
    inst.name = f"batch{i}"
    return inst


def batch4096(seed: int = 0, count: int = 4096, lo: int = 256, hi: int = 200_000,
              scale: float = 1.0, workers: int = 0) -> list[Instance]:
    """The batched workload: ``count`` independent mixture instances.

    ``workers`` > 1 generates the instances in a spawned process pool (each
    instance has its own seed, so the result does not depend on the pool)."""
    rng = _rng(seed)
    sizes = batch_sizes(rng, count, lo, hi)
    dims = np.where(rng.uniform(size=count) < 0.5, 2, 3)
    tasks = [(seed, i, max(int(sizes[i] * scale), 8), int(dims[i])) for i in range(count)]
    if workers > 1:
        import multiprocessing as mp
        from concurrent.futures import ProcessPoolExecutor
        with ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
            return list(ex.map(_batch_one, tasks, chunksize=16))
    return [_batch_one(t) for t in tasks]


def poisson_arrivals(seed: int, rate: float, duration: float) -> np.ndarray:
    rng = _rng(seed)
    t, out = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t >= duration:
            break
        out.append(t)
    return np.asarray(out)


def serve_stream(seed: int = 0, rate: float = 200.0, duration: float = 60.0,
                 pool: int = 512, lo: int = 1_000, hi: int = 2_000_000,
                 workers: int = 0) -> tuple[list[Instance], np.ndarray, np.ndarray]:
    """The served request stream: Poisson arrivals at ``rate`` per second for
    ``duration`` seconds, each request one mixture instance (2D/3D, sizes
    log-uniform in [lo, hi], eps the median 4th-NN distance, minpts in [4, 32]).

    Requests draw their instance uniformly from a pool of ``pool`` generated
    instances, so a long stream needs no more host memory than the pool.
    Returns (pool instances, arrival times in seconds, pool index per request)."""
    insts = batch4096(seed=seed + 1, count=pool, lo=lo, hi=hi, workers=workers)
    t = poisson_arrivals(seed + 2, rate, duration)
    which = _rng(seed + 3).integers(0, pool, size=t.shape[0])
    return insts, t, which


def write_csv(path: str, points: np.ndarray) -> None:
    """Write points in the reference's input format (no header, ',' separated)."""
    np.savetxt(path, points, delimiter=",", fmt="%.17g")


def tiny_cases() -> list[Instance]:
    """Hand-made edge cases (shared by the oracle tests and the GPU parity tests)."""
    cases = []
    # the reference's own fixture (test-datasets/ex.txt with common.h eps=1.5, minpts=3)
    ex = np.array([[1, 1], [2, 2], [3, 3], [10, 10], [11, 11], [12, 12],
                   [20, 20], [21, 21], [22, 22]], dtype=np.float64)
    cases.append(Instance(ex, 1.5, 3, "ex_txt"))
    # 3-4-5 triangle: d^2 == eps^2 exactly (inclusive boundary)
    tri = np.array([[0, 0], [3, 4], [6, 8], [9, 12], [100, 100]], dtype=np.float64)
    cases.append(Instance(tri, 5.0, 2, "eps_exact_345"))
    # duplicates
    dup = np.array([[1.0, 1.0]] * 6 + [[5.0, 5.0]] * 2 + [[1.2, 1.0]], dtype=np.float64)
    cases.append(Instance(dup, 0.5, 4, "duplicates"))
    # all noise
    r = _rng(7)
    cases.append(Instance(r.uniform(0, 1000, (200, 2)), 0.01, 3, "all_noise"))
    # a single dense cluster
    cases.append(Instance(r.normal(0, 0.1, (300, 2)), 0.5, 5, "single_cluster"))
    # minpts = 1: every point is core
    cases.append(Instance(r.uniform(0, 10, (150, 2)), 0.7, 1, "minpts1"))
    # fewer points than minpts
    cases.append(Instance(r.uniform(0, 1, (5, 2)), 0.3, 10, "n_lt_minpts"))
    # points on grid boundaries (multiples of eps/2) and at the bbox max
    g = np.array([[i * 0.25, j * 0.25] for i in range(9) for j in range(9)], dtype=np.float64)
    cases.append(Instance(g, 0.5, 5, "grid_boundaries"))
    # single point
    cases.append(Instance(np.array([[3.0, 4.0]]), 1.0, 1, "single_point"))
    # 3D small mixtures with borders shared between clusters
    r3 = _rng(11)
    pts3 = np.concatenate([r3.normal(0, 0.3, (400, 3)), r3.normal(1.2, 0.3, (400, 3)),
                           r3.uniform(-2, 3, (200, 3))])
    cases.append(Instance(pts3[r3.permutation(len(pts3))], 0.25, 6, "mix3d_small"))
    # two chains touching through one border point (border tie rule)
    chain = np.array([[0, 0], [0.5, 0], [1.0, 0], [1.5, 0], [2.0, 0],
                      [2.9, 0], [3.8, 0], [4.3, 0], [4.8, 0], [5.3, 0]], dtype=np.float64)
    cases.append(Instance(chain, 0.9, 3, "border_tie"))
    # negative and large-magnitude coordinates
    r4 = _rng(13)
    big = 1e4 + r4.normal(0, 1.0, (500, 2))
    big[::3] *= -1
    cases.append(Instance(big, 0.3, 4, "offset_coords"))
    return cases
