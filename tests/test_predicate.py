"""The exact-integer similarity predicate against the reference's long double
expression (CheckCoreCompSimCore) on exhaustive small grids and random large
values, including exact ties x == eps."""
import numpy as np
import pytest

from acctricnt_gb300 import accx
from oracle import oracle

EPS = [0.1, 0.15, 0.2, 0.25, 0.3, 1 / 3, 0.4, 0.5, 0.6, 2 / 3, 0.7, 0.75, 0.8, 0.9, 0.95, 1.0,
       0.0, -0.5, 1.5, 1e-12, np.nextafter(0.5, 0), np.nextafter(0.5, 1), 0.7071067811865476]


@pytest.mark.parametrize("eps", EPS)
def test_exhaustive_small_grid(eps):
    c, a, b = np.meshgrid(np.arange(2, 34), np.arange(1, 65), np.arange(1, 65), indexing="ij")
    c, a, b = c.ravel(), a.ravel(), b.ravel()
    ref = oracle.sim_batch(c, a, b, eps)
    got = accx.similar_exact_batch(c, a, b, eps)
    assert np.array_equal(ref, got)


@pytest.mark.parametrize("eps", [0.2, 0.5, 0.8, 0.3333, 0.123456789])
def test_random_large_values(eps):
    rng = np.random.default_rng(11)
    k = 200000
    du = rng.integers(1, 2_000_000, k)
    dv = rng.integers(1, 2_000_000, k)
    c = np.minimum(rng.integers(2, 2_000_000, k), np.minimum(du, dv) + 1)
    ref = oracle.sim_batch(c, du, dv, eps)
    got = accx.similar_exact_batch(c, du, dv, eps)
    assert np.array_equal(ref, got)


def test_exact_ties_and_near_ties():
    # x = cnn / sqrt(du*dv) equal to eps exactly (du*dv = (cnn/eps)^2) and one step either side
    rows = []
    for eps, cnn, du, dv in [(0.5, 2, 4, 4), (0.5, 3, 6, 6), (0.5, 5, 10, 10), (0.25, 2, 8, 8), (0.8, 4, 5, 5),
                             (0.75, 3, 4, 4), (0.6, 3, 5, 5), (0.2, 2, 10, 10), (0.5, 1000, 2000, 2000)]:
        for d in (-1, 0, 1):
            rows.append((eps, cnn, du, dv + d))
    for eps, cnn, du, dv in rows:
        assert accx.similar_exact(cnn, du, dv, eps) == bool(oracle.sim_batch([cnn], [du], [dv], eps)[0])
