"""Two-sample binomial agreement of per-detector / per-observable flip rates."""

import os

import numpy as np

RATES_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rates")


def rate_cases():
    return sorted(f[:-4] for f in os.listdir(RATES_DIR) if f.endswith(".npz"))


def load_rates(name):
    return dict(np.load(os.path.join(RATES_DIR, name + ".npz")))


def max_abs_z(c1, n1, c2, n2):
    """Largest |z| over bits of the two-proportion test (pooled variance); bits that never fire in
    either sample count as agreeing."""
    c1 = np.asarray(c1, dtype=np.float64)
    c2 = np.asarray(c2, dtype=np.float64)
    if c1.size == 0:
        return 0.0
    p = (c1 + c2) / (n1 + n2)
    var = p * (1 - p) * (1.0 / n1 + 1.0 / n2)
    diff = c1 / n1 - c2 / n2
    z = np.where(var > 0, np.abs(diff) / np.sqrt(np.where(var > 0, var, 1.0)), 0.0)
    return float(z.max())


def counts_from_packed(a, n):
    return np.unpackbits(a, axis=1, bitorder="little")[:, :n].sum(axis=0, dtype=np.int64)
