"""Seeded synthetic request streams for the benchmark and the tests.

* log-uniform group sizes (caller groups of a batch);
* Zipf(s) page ids over n items through a seeded random permutation, drawn
  by rejection-inversion (W. Hormann and G. Derflinger, "Rejection-inversion
  to generate variates from monotone discrete distributions", ACM TOMACS
  6(3), 1996), vectorised with numpy;
* geometric pin holds turned into per-round release lists (CSR);
* Poisson arrival times of the serving loop's tenants.
"""
from __future__ import annotations

import math

import numpy as np


def logu_counts(rng, shape, lo=1, hi=65536):
    """floor(exp(U(ln lo, ln(hi+1)))) clipped to [lo, hi]."""
    u = rng.uniform(math.log(lo), math.log(hi + 1), size=shape)
    return np.clip(np.floor(np.exp(u)), lo, hi).astype(np.int64)


class Zipf:
    """Zipf(s) on {1..n}: P(k) proportional to k^-s, rejection-inversion."""

    def __init__(self, n, s):
        assert n >= 1 and s > 0
        self.n, self.s = n, s
        self.h_x1 = self._H(1.5) - 1.0
        self.h_n = self._H(n + 0.5)
        self.cut = 2.0 - self._Hinv(self._H(2.5) - self._h(2.0))

    def _h(self, x):
        return np.exp(-self.s * np.log(x))

    def _H(self, x):
        # integral of h: (x^(1-s) - 1) / (1 - s), stable near s = 1
        lx = np.log(x)
        t = (1.0 - self.s) * lx
        return np.where(np.abs(t) > 1e-8, np.expm1(t) / np.where(t == 0, 1, t), 1.0 + t / 2) * lx

    def _Hinv(self, x):
        t = x * (1.0 - self.s)
        return np.exp(np.where(np.abs(t) > 1e-8, np.log1p(t) / np.where(t == 0, 1, t), 1.0 - t / 2) * x)

    def sample(self, rng, size):
        out = np.empty(size, dtype=np.int64)
        filled = 0
        while filled < size:
            m = int((size - filled) * 1.1) + 16
            u = self.h_n + rng.uniform(size=m) * (self.h_x1 - self.h_n)
            x = self._Hinv(u)
            k = np.clip(np.floor(x + 0.5), 1, self.n)
            ok = (k - x <= self.cut) | (u >= self._H(k + 0.5) - self._h(k))
            acc = k[ok].astype(np.int64)
            take = min(len(acc), size - filled)
            out[filled:filled + take] = acc[:take]
            filled += take
        return out


def zipf_pages(n_items, s, count, seed, chunk=1 << 22):
    """`count` page ids: Zipf(s) ranks mapped through a seed-permuted table."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(n_items).astype(np.int32)
    z = Zipf(n_items, s)
    out = np.empty(count, dtype=np.int32)
    for a in range(0, count, chunk):
        b = min(count, a + chunk)
        out[a:b] = perm[z.sample(rng, b - a) - 1]
    return out


def release_lists(n_rounds, round_size, p_hold, seed):
    """Each fetch of round r keeps its pin for h ~ Geometric(p) >= 1 rounds and
    is released at the start of round r + h.  Returns CSR (ptr[n_rounds+1],
    idx) of global fetch indices released per round (releases past the last
    round are dropped)."""
    rng = np.random.default_rng(seed)
    total = n_rounds * round_size
    holds = rng.geometric(p_hold, size=total)
    rel_round = np.repeat(np.arange(n_rounds), round_size) + holds
    keep = rel_round < n_rounds
    idx = np.nonzero(keep)[0]
    rr = rel_round[keep]
    # small-range key: numpy's stable sort is a radix sort for 16-bit integers
    key = rr.astype(np.uint16) if n_rounds <= 65535 else rr
    order = np.argsort(key, kind="stable")
    idx = idx[order].astype(np.int32)
    counts = np.bincount(rr[order], minlength=n_rounds)
    ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    return ptr, idx


def poisson_arrivals(rng, rate_per_s, horizon_s):
    """Arrival times (seconds) of a Poisson process on [0, horizon)."""
    n = rng.poisson(rate_per_s * horizon_s)
    return np.sort(rng.uniform(0.0, horizon_s, size=n))
