"""The kernels' environment light sampling by alias tables, restated on the CPU.

`pick_light` (device_shading.cuh) picks a row, then a column, each from a 24-bit draw u = k 2^-24:
bin (k n) >> 24, the rest of k n as the in-texel fraction, and a keep-or-alias decision against
the table entry by a separate uniform that is rescaled after each decision. The tables come from
the package's builder (`alias_table`, host_common.h), exported by the oracle library. Here:
  * every one of the 2^24 draws of one decision, enumerated: the realised bin probabilities equal
    the weights' within the 24-bit resolution (a bin collects a few 2^-24 steps of error per
    table entry that aliases to it);
  * the chained 2D pick on a small environment by Monte Carlo: texel frequencies within sampling
    noise of the density, in-texel fractions uniform.
"""
import numpy as np

from oracle import binding as O

STEP = np.float32(5.9604644775390625e-08)  # 2^-24


def _bin_of(u, n):
    kn = (u * np.float32(16777216.0)).astype(np.uint64) * np.uint64(n)
    return (kn >> np.uint64(24)).astype(np.int64), (kn & np.uint64(0xFFFFFF)).astype(np.float32) * STEP


def _alias_pick(entries, i, d):
    """Bin i (its table entries given) kept or replaced by its alias, and d rescaled."""
    p = np.ascontiguousarray(entries[:, 0]).view(np.float32)
    keep = d < p
    with np.errstate(divide="ignore", invalid="ignore"):
        d2 = np.where(keep, d / p, (d - p) / (np.float32(1) - p)).astype(np.float32)
    return np.where(keep, i, entries[:, 1].astype(np.int64)), d2


def _weights(rng, n):
    w = rng.lognormal(0.0, 2.0, n)
    w[rng.integers(0, n, n // 10)] *= 1e-4
    return w


def test_alias_table_exact_enumeration():
    rng = np.random.default_rng(3)
    for n in (7, 1000, 1024):
        w = _weights(rng, n)
        t = O.alias_table(w)
        p = w / w.sum()
        # the table encodes the distribution exactly (up to the float keep probabilities)
        keep = t[:, 0].view(np.float32).astype(np.float64)
        enc = keep / n
        np.add.at(enc, t[:, 1].astype(np.int64), (1.0 - keep) / n)
        assert np.abs(enc - p).max() < 1e-7  # keep probabilities stored as float
        # every 24-bit bin draw with every 24-bit decision draw of its bin's share
        k = np.arange(1 << 24, dtype=np.uint64)
        i = (k * np.uint64(n) >> np.uint64(24)).astype(np.int64)
        d = ((k * np.uint64(n)) & np.uint64(0xFFFFFF)).astype(np.float32) * STEP
        out, _ = _alias_pick(t[i], i, d)
        got = np.bincount(out, minlength=n) / float(1 << 24)
        indeg = np.bincount(t[:, 1].astype(np.int64), minlength=n) + 1
        assert np.all(np.abs(got - p) <= indeg * (n / float(1 << 24)) * 1.01 + 1e-12), n
        assert abs(got.sum() - 1.0) < 1e-12


def test_env_pick_2d_density_and_fractions():
    rng = np.random.default_rng(11)
    H, W = 16, 24
    f = rng.lognormal(0.0, 1.5, (H, W))
    f[rng.random((H, W)) < 0.1] *= 1e-3
    rows = O.alias_table(f.sum(1))
    cols = np.stack([O.alias_table(f[y]) for y in range(H)])
    N = 4_000_000
    u0, u1, u2 = (rng.integers(0, 1 << 24, N).astype(np.float32) * STEP for _ in range(3))
    d = u0.copy()  # the strategy draw, rescaled by p_env = 1
    b, fy = _bin_of(u1, H)
    y, d = _alias_pick(rows[b], b, d)
    b2, fx = _bin_of(u2, W)
    x, _ = _alias_pick(cols[y, b2], b2, d)
    cnt = np.bincount(y * W + x, minlength=H * W).reshape(H, W) / N
    P = f / f.sum()
    z = (cnt - P) / np.sqrt(P * (1 - P) / N)
    assert np.abs(z).max() < 5.0 and (z ** 2).mean() < 1.5
    for frac in (fx, fy):
        assert abs(frac.mean() - 0.5) < 2e-3 and abs(frac.var() - 1 / 12) < 2e-3
