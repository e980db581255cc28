"""Small shared helpers for the test suite."""
import numpy as np


def rel(a, b):
    """max |a - b| / max |b| (0 if both vanish)."""
    a, b = np.asarray(a), np.asarray(b)
    d = np.abs(a - b).max()
    s = np.abs(b).max()
    return 0.0 if d == 0 else d / (s if s > 0 else 1.0)


def rand_spec(T, nb, seed=1, slope=0.0):
    from gdpy import inputs

    rng = np.random.default_rng(seed)
    deg, order = inputs.degree_order(T)
    a = rng.standard_normal((nb, deg.size)) + 1j * rng.standard_normal((nb, deg.size))
    a[:, order == 0] = a[:, order == 0].real
    if slope:
        a *= np.maximum(deg, 1).astype(float) ** slope
    return a
