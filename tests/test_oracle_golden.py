"""The oracle (CPU restatement) against fixtures produced by the reference's own
CPU build: counts, similarity, labels, clusters and the result-file bytes."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, load_golden
from oracle import oracle


def plain_config_digests():
    """sha256 digests of the reference build's outputs on the plain CPU config:
    R-MAT scale 16, edge factor 16, seed 1, eps 0.2, mu 5."""
    with open(os.path.join(GOLDEN, "rmat16_e02_mu5_digests.json")) as f:
        return json.load(f)


def sha256(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


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


def test_oracle_matches_reference_on_the_plain_cpu_config(tmp_path):
    """R-MAT scale 16 (65,536 vertices, 1.82M entries), eps 0.2, mu 5: every
    output of the oracle has the digest of the reference build's output."""
    from acctricnt_gb300 import accx
    fx = plain_config_digests()
    off, dst = accx.generate_host(accx.rmat_params(16, 16, seed=1))
    assert sha256(off) == fx["graph_sha256"]["off"] and sha256(dst) == fx["graph_sha256"]["dst"]
    r = oracle.scan(off, dst, fx["eps"], fx["mu"], nthreads=4, out_dir=str(tmp_path))
    for k in ("cnn", "sim", "label", "cluster"):
        assert sha256(r[k]) == fx["sha256"][k], k
    with open(os.path.join(str(tmp_path), fx["result_name"]), "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == fx["result_sha256"]
