"""The request server (continuous batching): each request's result is the same
alone and in a concurrent mix, equals the CPU oracle, and admission keeps held
device memory within the HBM budget."""
import numpy as np
import pytest

from conftest import has_gpu

pytestmark = pytest.mark.gpu

if has_gpu():
    from acctricnt_gb300 import accx
    from oracle import oracle

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _mix(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15))
    x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def _query_digest(label, cluster):
    u = np.arange(len(label), dtype=np.uint64)
    key = (u << np.uint64(34)) ^ (label.astype(np.uint64) << np.uint64(32)) ^ cluster.astype(np.uint32).astype(np.uint64)
    with np.errstate(over="ignore"):
        return int(_mix(key).sum(dtype=np.uint64))


def _count_digest(cnt):
    e = np.arange(len(cnt), dtype=np.uint64)
    with np.errstate(over="ignore"):
        return int(cnt.astype(np.uint64).sum()), int(_mix((e << np.uint64(32)) | cnt.astype(np.uint32).astype(np.uint64)).sum(dtype=np.uint64))


def _requests(seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(36):
        if i % 6 == 5:
            reqs.append(accx.count_request(accx.rmat_params(int(rng.integers(10, 15)), 16, seed=100 + i)))
        else:
            reqs.append(accx.query_request(float(rng.uniform(0.1, 0.9)), int(rng.integers(2, 21))))
    return reqs


def _key(r):
    s = r.summary
    return (r.status, r.type, s.cores, s.clusters, s.hubs, s.outliers, s.similar_entries, s.digest, r.n, r.m,
            r.count_sum, r.count_digest)


def test_results_identical_alone_and_in_the_mix_and_equal_the_oracle():
    G = accx.Graph.generate(accx.rmat_params(16, 16, seed=3))
    G.relabel()
    G.count(policy="bitmap", out=None)
    reqs = _requests(1)
    alone = accx.Server(G, workers=1)
    res_alone = [_key(alone.wait(alone.submit(r))) for r in reqs]
    alone.close()
    mix = accx.Server(G, workers=6)
    ids = [mix.submit(r) for r in reqs]
    res_mix = [_key(mix.wait(i)) for i in ids]
    st = mix.stats()
    mix.close()
    assert res_alone == res_mix
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["max_concurrent"] >= 2  # requests really ran at the same time
    off, dst = G.download()
    cnn = oracle.cn_count(off, dst, nthreads=8)
    for r, k in zip(reqs, res_mix):
        if r.type == accx.REQ_QUERY:
            sim, _, lab0 = oracle.similarity(off, dst, cnn, r.eps, r.mu)
            lab, cl = oracle.cluster(off, dst, sim, lab0)
            assert k[7] == _query_digest(lab, cl)
            assert k[2] == int((lab == 1).sum()) and k[4] == int((lab == 2).sum())
        else:
            o2, d2 = accx.generate_host(r.graph)
            c2 = oracle.cn_count(o2, d2, nthreads=8) - 2
            assert (k[8], k[9]) == (len(o2) - 1, len(d2))
            assert (k[10], k[11]) == _count_digest(c2)


def test_admission_respects_the_hbm_budget():
    G = accx.Graph.generate(accx.rmat_params(12, 16, seed=4))
    G.count(policy="heuristic", out=None)
    reqs = [accx.count_request(accx.rmat_params(14, 16, seed=200 + i)) for i in range(8)]
    per = accx.Server(G, workers=1).request_bytes(reqs[0])
    budget = int(per * 2.5)  # room for two at a time
    S = accx.Server(G, workers=8, hbm_budget=budget)
    ids = [S.submit(r) for r in reqs]
    out = [S.wait(i) for i in ids]
    st = S.stats()
    S.close()
    assert all(r.status == 0 for r in out)
    assert st["peak_bytes"] <= budget
    assert st["max_concurrent"] >= 2


def test_oriented_count_requests_equal_direct_counts():
    """count_orient: count requests relabel their graph and count oriented; the
    digests equal those of the CPU oracle's counts, alone and in a mix."""
    G = accx.Graph.generate(accx.rmat_params(12, 16, seed=5))
    G.count(policy="heuristic", out=None)
    reqs = [accx.count_request(accx.rmat_params(11 + i % 4, 16, seed=300 + i)) for i in range(8)]
    plain = accx.Server(G, workers=1)
    per_direct = plain.request_bytes(reqs[0])
    plain.close()
    S = accx.Server(G, workers=4, count_orient=True)
    assert S.request_bytes(reqs[0]) > per_direct  # relabel + oriented scratch admitted
    ids = [S.submit(r) for r in reqs]
    out = [S.wait(i) for i in ids]
    S.close()
    for r, res in zip(reqs, out):
        assert res.status == 0
        o2, d2 = accx.generate_host(r.graph)
        c2 = oracle.cn_count(o2, d2, nthreads=8) - 2
        assert (res.count_sum, res.count_digest) == _count_digest(c2)
