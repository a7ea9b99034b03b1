"""CPU checks of the bench's measurement helpers (no GPU).

The CPU baseline times every stride-th owner (in modelled-work order) of the
oracle port of CheckCoreBitmap and scales by the sampled share of the work; the
samples for starts 0..stride-1 must partition the owners, so that together they
reproduce the whole count exactly and their work shares sum to one.
"""
import numpy as np
import pytest

import bench
from acctricnt_gb300 import accx
from oracle import oracle


@pytest.mark.parametrize("stride", [1, 3, 7])
def test_sampler_strides_partition_the_whole_count(stride):
    off, dst = accx.generate_host(accx.rmat_params(12, 16, seed=3))
    full = oracle.cn_count(off, dst, 2)
    cs = bench.CpuSampler(off, dst, 2)
    frac, owned = 0.0, 0
    for start in range(stride):
        r = cs.run(stride, start=start)
        frac += r["frac"]
        owned += r["owned"]
        assert r["full_s"] >= r["dt"]
    assert np.array_equal(cs.cnn[:len(dst)], full)
    assert owned == len(dst) // 2  # every undirected edge has one owner
    assert frac == pytest.approx(1.0)


def test_sampler_orders_owners_by_modelled_work():
    off, dst = accx.generate_host(accx.rmat_params(11, 16, seed=4))
    cs = bench.CpuSampler(off, dst, 1)
    assert np.all(np.diff(cs.cost[cs.order]) >= 0)
    assert cs.total == pytest.approx(float(oracle.owner_costs(off, dst, 1).sum()))


def test_measured_regret():
    assert bench.measured_regret(10.0, {"a": 12.0, "b": 9.0}) == {"best": "b", "best_ms": 9.0, "frac": 0.1111}
    assert bench.measured_regret(8.0, {"a": 12.0}) == {"best": "model", "best_ms": 8.0, "frac": 0.0}
