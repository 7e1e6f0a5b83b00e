"""Seeded synthetic inputs shared by the parity tests."""
import numpy as np

W9 = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
W15 = np.array([2 / 9] + [1 / 9] * 6 + [1 / 72] * 8)


def weights(q):
    return W9 if q == 9 else W15


def pops(rng, q, n, amp=0.1, base=1.0):
    w = weights(q)[:, None]
    return np.ascontiguousarray(w * base * (1.0 + amp * rng.standard_normal((q, n))))


def field(rng, n, lo, hi):
    return np.ascontiguousarray(rng.uniform(lo, hi, n))
