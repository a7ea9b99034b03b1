"""Seeded synthetic workloads used by the bench and the tests.

They stand in for the reference's R-MAT/SNAP inputs (not shipped); every graph
is produced by the counter-based generators of libaccx, so a seed names a graph.
"""
import numpy as np

from . import accx


def rmat24():
    """R-MAT scale 24, edge factor 16, (0.57, 0.19, 0.19, 0.05), seed 1."""
    return accx.rmat_params(24, 16, seed=1)


def chung_lu_20m():
    """Chung-Lu, 20M vertices, exponent 2.1, mean degree 24, max expected degree 1M."""
    return accx.chung_lu_params(20_000_000, 24, 2.1, 1e6, seed=1)


def er_20m():
    """Erdos-Renyi, 20M vertices, mean degree 24."""
    return accx.er_params(20_000_000, 24, seed=1)


def batch_uneven(k=512, seed=1, emin=1e3, emax=2e6):
    """K graphs with undirected edge draws log-uniform in [emin, emax]: a seeded
    mix of R-MAT (scale 10-18, edge factor set to reach the draw count) and
    Erdos-Renyi (mean degree 16) graphs."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(k):
        e = int(np.exp(rng.uniform(np.log(emin), np.log(emax))))
        s = seed * 1_000_003 + i
        if rng.random() < 0.5:
            scale = int(np.clip(round(np.log2(max(e / 16.0, 1.0))), 10, 18))
            ef = max(1, int(round(e / float(1 << scale))))
            out.append(accx.rmat_params(scale, ef, seed=s))
        else:
            n = max(64, e // 8)
            out.append(accx.gen_params(accx.GEN_ER, n, e, seed=s))
    return out
