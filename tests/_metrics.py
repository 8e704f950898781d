"""Adjusted Rand index in numpy (scikit-learn is not installed on every test
machine).  Noise (-1) is treated as its own label, as sklearn does."""
import numpy as np


def _comb2(x):
    x = np.asarray(x, dtype=np.float64)
    return x * (x - 1) / 2.0


def adjusted_rand_score(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    _, ai = np.unique(a, return_inverse=True)
    _, bi = np.unique(b, return_inverse=True)
    n = a.shape[0]
    table = np.zeros((ai.max() + 1, bi.max() + 1), dtype=np.int64)
    np.add.at(table, (ai, bi), 1)
    sum_comb = _comb2(table).sum()
    sa = _comb2(table.sum(axis=1)).sum()
    sb = _comb2(table.sum(axis=0)).sum()
    expected = sa * sb / _comb2(n) if n > 1 else 0.0
    mx = (sa + sb) / 2.0
    if mx == expected:
        return 1.0
    return float((sum_comb - expected) / (mx - expected))
