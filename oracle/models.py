"""Closed-form step-count models for random-walk page allocation.

TEST INFRASTRUCTURE ONLY: used by the statistical parity tests as the
expected mean number of steps per request.  Restated from the reference's
``theoretical_models.py`` (lines cited per function); the restatement is
pinned against that module's own outputs by ``tests/golden/model_predictions.json``
(generated by ``tests/golden/make_model_fixtures.py``).

Notation: T pages in the pool, A free pages before the batch, N requests.
"TAS" = mean steps per thread, "WAS" = mean over warps of the per-warp
maximum (unitTests/metrics.h:13-33).
"""
from __future__ import annotations

import math

import numpy as np


def queue_tas(T, A, N):
    """theoretical_models.py:12-13"""
    return (N + 1) / 2


def queue_was(T, A, N):
    """theoretical_models.py:16-17"""
    return 32 / 33 * N


def rw_tas(T, A, N):
    """Page-probe walk: theoretical_models.py:20-21, T/N * ln(A/(A-N))."""
    return T / N * math.log(A / (A - N))


def _sum_until_small(term, k0=0, tol=1e-16, kmax=10**7, chunk=4096):
    """Sum term(k) for k = k0, k0+1, ... (vectorised) until a whole chunk of
    terms is below tol, or kmax terms.  The reference sums 10^7 terms; the
    terms here are monotone decreasing, so the tail dropped is below tol*chunk."""
    s = 0.0
    k = k0
    while k < kmax:
        ks = np.arange(k, min(k + chunk, kmax), dtype=np.float64)
        t = term(ks)
        s += float(t.sum())
        if t[-1] < tol:
            break
        k += chunk
    return s


def rw_was(T, A, N):
    """Per-warp maximum of the page-probe walk: theoretical_models.py:24-31."""
    q = (T - A + N) / T
    return _sum_until_small(lambda k: 1.0 - (1.0 - q ** k) ** 32)


def rwbm_tas(T, A, N):
    """Word-probe walk over a 32-bit bitmap: theoretical_models.py:34-41."""
    k = np.arange(0, N - 1, dtype=np.float64)
    return float((1.0 / (1.0 - ((T - A + k) / T) ** 32) / N).sum())


def rwbm_was(T, A, N):
    """theoretical_models.py:44-51"""
    q = (T - A + N) / T
    return _sum_until_small(lambda k: 1.0 - (1.0 - q ** (32 * k)) ** 32)


def corwbm_was(T, A, N):
    """Warp-collaborative walk, warp steps: theoretical_models.py:54-62."""
    import mpmath

    mpmath.mp.dps = 100
    mu = 1024 * (A - N) / T
    sigma = 1024 * (A - N) / T * (T - A + N) / T
    eb = mpmath.quad(
        lambda t: 32 / (sigma * math.sqrt(2 * math.pi * t))
        * math.exp(-(32 - mu * t) ** 2 / (2 * (sigma ** 2) * t)),
        [0, mpmath.inf],
    )
    return max(1, float(eb))


def rwbm64_tas(T, A, N):
    """Word-probe walk over 64-bit words: the 32-bit model with 64 bits per
    word (same derivation, theoretical_models.py:34-41)."""
    k = np.arange(0, N - 1, dtype=np.float64)
    return float((1.0 / (1.0 - ((T - A + k) / T) ** 64) / N).sum())
