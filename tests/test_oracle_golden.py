"""The oracle (CPU restatement) against fixtures produced by the reference's own
CPU build: counts, similarity, labels, clusters and the result-file bytes."""
import os

import numpy as np
import pytest

from conftest import golden_cases, load_golden
from oracle import oracle


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference(name, tmp_path):
    g = load_golden(name)
    off, dst = g["off"], g["dst"]
    assert oracle.check_graph(off, dst) == 0
    r = oracle.scan(off, dst, float(g["eps"]), int(g["mu"]), out_dir=str(tmp_path))
    assert np.array_equal(r["cnn"], g["cnn"])
    assert np.array_equal(r["sim"], g["sim"])
    assert np.array_equal(r["label"], g["label"])
    assert np.array_equal(r["cluster"], g["cluster"])
    with open(os.path.join(str(tmp_path), str(g["result_name"])), "rb") as f:
        assert f.read() == g["result"].tobytes()


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_count_thread_independent(name):
    g = load_golden(name)
    assert np.array_equal(oracle.cn_count(g["off"], g["dst"], nthreads=4), g["cnn"])


def test_oracle_rejects_bad_graphs():
    off = np.array([0, 1, 2], np.uint32)
    assert oracle.check_graph(off, np.array([0, 0], np.int32)) == -1  # self loop
    off = np.array([0, 2, 3, 4], np.uint32)
    assert oracle.check_graph(off, np.array([2, 1, 0, 0], np.int32)) == -2  # unsorted row
    assert oracle.check_graph(off, np.array([1, 7, 0, 0], np.int32)) == -3  # out of range
