"""Batches of uneven graphs: one count / one SCAN query over the disjoint union
equals every graph's own results; the CUDA-graph-captured count equals the eager
one; the autotuner's launch shape gives identical counts."""
import numpy as np
import pytest

from conftest import golden_cases, has_gpu, load_golden

pytestmark = pytest.mark.gpu

if has_gpu():
    from acctricnt_gb300 import accx, workloads


def _graphs():
    gs, refs = [], []
    for name in golden_cases():
        g = load_golden(name)
        gs.append(accx.Graph.from_csr(g["off"], g["dst"]))
        refs.append(g)
    for p in workloads.batch_uneven(k=12, seed=5, emin=500, emax=60000):
        gs.append(accx.Graph.generate(p))
        refs.append(None)
    return gs, refs


def test_union_count_and_scan_equal_per_graph_results():
    gs, refs = _graphs()
    B = accx.Batch(gs)
    U = B.union
    cnt = U.count(policy="heuristic", bias=2)
    for G, g, c in zip(gs, refs, B.split(cnt)):
        want = g["cnn"] if g is not None else G.count(policy="bitmap", bias=2)
        assert np.array_equal(c, want)
    U.relabel()
    assert np.array_equal(U.count(policy="bitmap", bias=2), cnt)
    r = U.scan(0.3, 4)
    for (vb, n, eb, m), G, lab, cl in zip(B.ranges, gs, B.split(r["label"], per="vertex"),
                                          B.split(r["cluster"], per="vertex")):
        G.count(policy="heuristic", out=None)
        rg = G.scan(0.3, 4)
        assert np.array_equal(lab, rg["label"])
        assert np.array_equal(np.where(cl >= 0, cl - vb, -1), rg["cluster"])


def test_captured_replay_matches_eager():
    import torch
    gs, _ = _graphs()
    B = accx.Batch(gs)
    U = B.union
    U.relabel()
    want = U.count(policy="bitmap", bias=2)
    s = torch.cuda.Stream()
    B.capture(policy="bitmap", bias=2, stream=s.cuda_stream)
    for _ in range(3):
        U.count(policy="merge", bias=7, out=None)  # leave different values resident
        torch.cuda.synchronize()
        B.launch(stream=s.cuda_stream)
        s.synchronize()
        assert np.array_equal(U.read_counts(), want)


def test_autotuned_shape_counts_identically():
    G = accx.Graph.generate(accx.rmat_params(17, 16, seed=8))
    G.relabel()
    want = G.count(policy="bitmap")
    kw, ms, allms = G.autotune(policy="bitmap", reps=1)
    assert ms > 0 and len(allms) >= 7
    assert np.array_equal(G.count(policy="bitmap", **kw), want)


def test_oriented_capture_and_autotune_match_eager():
    """Oriented counts in a captured batch replay and under the oriented
    autotuner's launch shape equal the eager direct counts."""
    import torch
    gs, _ = _graphs()
    B = accx.Batch(gs)
    U = B.union
    U.relabel()
    want = U.count(policy="bitmap", bias=2)
    s = torch.cuda.Stream()
    kw, ms, allms = U.autotune(policy="bitmap", reps=1, stream=s.cuda_stream, orient=True)
    assert ms > 0 and kw["window_kb"] in (0, 32, 40, 48, 56, 64, 80)  # 0: the library's default shape
    B.capture(policy="bitmap", bias=2, stream=s.cuda_stream, orient=True, **kw)
    for _ in range(2):
        U.count(policy="merge", bias=7, out=None)
        torch.cuda.synchronize()
        B.launch(stream=s.cuda_stream)
        s.synchronize()
        assert np.array_equal(U.read_counts(), want)


def test_bench_batch_against_the_oracle(default_sched):
    """The batch workload exactly as the bench runs it -- 512 graphs, undirected
    edge draws log-uniform 1K-2M, R-MAT scale 10-18 / ER mix, seed 1 -- counted
    as one captured oriented launch under the scheduler's model: every graph's
    slice of the union counts equals the oracle's CheckCoreBitmap on that graph."""
    import torch
    from oracle import oracle
    gs = [accx.Graph.generate(p) for p in workloads.batch_uneven(k=512, seed=1)]
    B = accx.Batch(gs)
    U = B.union
    U.relabel()
    U.set_model(default_sched.model(True), orient=True)
    s = torch.cuda.Stream()
    B.capture(policy="model", bias=2, stream=s.cuda_stream, orient=True)
    B.launch(stream=s.cuda_stream)
    s.synchronize()
    for i, (G, c) in enumerate(zip(gs, B.split(U.read_counts()))):
        off, dst = G.download()
        assert np.array_equal(c, oracle.cn_count(off, dst, nthreads=0)), i
