"""CPU checks of the bench's measurement helpers (no GPU).

The CPU baseline and the reference arm time stripes of the reference's
CheckCoreBitmap entry chunks (restated in the oracle): the K stripes of a count
must partition its entries and together give exactly the whole count, in the
original vertex order and in the reference's degree-descending order.
"""
import numpy as np
import pytest

import bench
from acctricnt_gb300 import accx
from oracle import oracle


@pytest.mark.parametrize("k", [1, 3, 20])
def test_stripes_partition_the_whole_count(k):
    off, dst = accx.generate_host(accx.rmat_params(12, 16, seed=3))
    full = oracle.cn_count(off, dst, 2)
    for name, (o, d) in bench.cpu_orders(off, dst, 2).items():
        cnn = np.full(len(d), 2, np.int32)
        entries, secs = bench.time_stripes(o, d, cnn, bench.spread_stripes(k), k, 2)
        assert entries == len(d) and len(secs) == k
        if name == "none":
            assert np.array_equal(cnn, full)
        else:
            assert np.array_equal(cnn, oracle.cn_count(o, d, 2))
            assert cnn.sum(dtype=np.int64) == full.sum(dtype=np.int64)


def test_stripe_budget_stops_early_but_counts_whole_stripes():
    off, dst = accx.generate_host(accx.rmat_params(11, 16, seed=4))
    cnn = np.full(len(dst), 2, np.int32)
    entries, secs = bench.time_stripes(off, dst, cnn, bench.spread_stripes(8), 8, 1, budget_s=0.0)
    assert len(secs) == 1
    assert 0 < entries < len(dst)


@pytest.mark.parametrize("k", [1, 2, 5, 8, 20])
def test_spread_stripes_is_a_permutation_spread_over_the_count(k):
    order = bench.spread_stripes(k)
    assert sorted(order) == list(range(k))
    if k >= 4:
        assert order[:2] == [0, k // 2]


def test_reorder_deg_is_the_degree_descending_relabel():
    off, dst = accx.generate_host(accx.chung_lu_params(3000, 10, 2.1, 300, seed=5))
    no, nd, old = oracle.reorder_deg(off, dst, 2)
    deg = np.diff(off.astype(np.int64))
    ndeg = np.diff(no.astype(np.int64))
    assert np.array_equal(ndeg, deg[old]) and np.all(np.diff(ndeg) <= 0)
    assert sorted(old.tolist()) == list(range(len(off) - 1))
    assert oracle.check_graph(no, nd) == 0
    new = np.empty_like(old)
    new[old] = np.arange(len(old), dtype=old.dtype)
    src = np.repeat(np.arange(len(off) - 1), np.diff(off.astype(np.int64)))
    mapped = set(zip(new[src].tolist(), new[dst].tolist()))
    rsrc = np.repeat(np.arange(len(no) - 1), np.diff(no.astype(np.int64)))
    assert mapped == set(zip(rsrc.tolist(), nd.tolist()))


def test_both_arms_print_the_same_config():
    class A:
        scale, edge_factor = 24, 16
    assert bench.workload_config(A, 10, 20, 1) == bench.workload_config(A, 10, 20, 1)
    assert "R-MAT scale 24" in bench.workload_config(A, 10, 20, 1)["workload"]


def test_measured_regret():
    assert bench.measured_regret(10.0, {"a": 12.0, "b": 9.0}) == {"best": "b", "best_ms": 9.0, "frac": 0.1111}
    assert bench.measured_regret(8.0, {"a": 12.0}) == {"best": "model", "best_ms": 8.0, "frac": 0.0}
