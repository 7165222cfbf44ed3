"""Float32 cell keys: the bound that lets k_keys take a cell from float32
arithmetic must make it equal to the float64 cell.

k_keys computes t64 = fl64(fl64(x - lo) * inv_f) and floor(t64).  Its float32
path uses x32 = x rounded toward zero (from the bits), lo32 = fl32(lo),
i32 = fl32(inv_f) and t32 = fl32(fl32(x32 - lo32) * i32), and takes floor(t32)
when t32 is farther than key_band from every integer.  key_band is set per
instance in k_params_inst:

    1.25 ((maxabs 2^-23 + |lo| 2^-24) inv_f (1 + 2^-22) + (G + 1)(3 2^-24 + 2^-47))

This test restates both paths with IEEE float32/float64 numpy arithmetic (no
GPU) over random, boundary-hugging and far-from-origin coordinates and checks
floor(t32) == floor(t64) wherever the float32 path would be taken."""
import numpy as np


def _rz32(x):
    """float64 -> float32 rounded toward zero (the bit truncation k_keys uses)."""
    f = x.astype(np.float32)                       # round to nearest
    over = np.abs(f.astype(np.float64)) > np.abs(x)
    f[over] = np.nextafter(f[over], np.float32(0))
    return f


def _band(lo, hi, inv_f, G):
    maxabs = max(np.max(np.abs(lo)), np.max(np.abs(hi)))
    loabs = np.max(np.abs(lo))
    gmax = max(1.0, float(np.max(G)))
    b = 1.25 * ((maxabs * 2.0 ** -23 + loabs * 2.0 ** -24) * inv_f * (1 + 2.0 ** -22)
                + (gmax + 1.0) * (3 * 2.0 ** -24 + 2.0 ** -47))
    b32 = np.float32(b)
    if float(b32) < b:
        b32 = np.nextafter(b32, np.float32(np.inf))
    return b, b32


def _check(points, eps, mult=0.5 * (1 + 2.0 ** -16)):
    lo, hi = points.min(axis=0), points.max(axis=0)
    f = eps * mult
    inv_f = 1.0 / f
    G = np.floor((hi - lo) * inv_f) + 1
    band, b32 = _band(lo, hi, inv_f, G)
    if not (band < 0.125 and G.max() < 2 ** 21):
        return 0                                    # the float32 path is off
    t64 = (points - lo) * inv_f                     # two float64 roundings, as on the device
    q64 = np.floor(t64)
    x32 = _rz32(points)
    t32 = (x32 - lo.astype(np.float32)) * np.float32(inv_f)
    assert t32.dtype == np.float32
    fl = np.floor(t32)
    fr = t32 - fl
    fast = (np.abs(t32) < np.float32(4194304.0)) & (fr > b32) & (fr < np.float32(1) - b32)
    bad = fast & (fl.astype(np.float64) != q64)
    assert not bad.any(), (points[bad][:4], t64[bad][:4], t32[bad][:4], band)
    return int(fast.sum())


def test_random_and_far_from_origin():
    rng = np.random.default_rng(5)
    taken = 0
    for scale, offset, eps in [(1000.0, 0.0, 0.3), (10.0, 0.0, 0.05), (1.0, 0.0, 1e-3),
                               (1e4, 5e5, 2.0), (100.0, -3e3, 0.01), (1e-3, 1.0, 1e-6),
                               (50.0, 0.0, 0.7)]:
        for d in (2, 3):
            pts = offset + rng.uniform(0, scale, (200_000, d))
            taken += _check(pts, eps)
    assert taken > 1_000_000          # the fast path is taken for most coordinates


def test_coordinates_next_to_cell_boundaries():
    rng = np.random.default_rng(6)
    for eps, span in [(0.3, 1000.0), (0.05, 10.0), (2.0, 3e4)]:
        f = eps * 0.5 * (1 + 2.0 ** -16)
        # exact boundary positions lo + c f and their float64 neighbours
        lo = 0.0
        c = rng.integers(1, int(span / f) - 1, 50_000).astype(np.float64)
        b = lo + c * f
        off = rng.choice([-3, -2, -1, 0, 1, 2, 3], size=b.shape).astype(np.float64)
        x = b + off * np.spacing(b) + rng.normal(0, 1e-9 * f, b.shape)
        pts = np.stack([x, rng.uniform(0, span, b.shape)], axis=1)
        pts = np.concatenate([pts, [[0.0, 0.0], [span, span]]])
        _check(pts, eps)
