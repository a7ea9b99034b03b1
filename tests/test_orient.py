"""GPU parity of oriented counting (triangle credits on prefix lists): the same
counts as the reference and the oracle, under every policy, with and without the
degree-descending relabel, and with windows and owner counters small enough
that bitmap owners fall back to merge."""
import numpy as np
import pytest

from conftest import golden_cases, has_gpu, load_golden

pytestmark = pytest.mark.gpu

if has_gpu():
    from acctricnt_gb300 import accx
    from oracle import oracle

POLICIES = ["heuristic", "merge", "gallop", "bitmap"]


def _table(seed):
    rng = np.random.default_rng(seed)
    return rng.integers(0, 3, size=(24, 24)).astype(np.uint8)


def _all_orient(G, ref, bias=2):
    for pol in POLICIES:
        assert np.array_equal(G.count(policy=pol, bias=bias, orient=True), ref), pol
    assert np.array_equal(G.count(policy="table", table=_table(3), bias=bias, orient=True), ref)
    # an 8192-id window and 256 owner counters: most bitmap owners fall back to galloping
    assert np.array_equal(G.count(policy="bitmap", bias=bias, orient=True, window_kb=1, sparse_kb=1,
                                  block_warps=4), ref)


@pytest.mark.parametrize("name", golden_cases())
def test_orient_golden(name):
    g = load_golden(name)
    G = accx.Graph.from_csr(g["off"], g["dst"])
    _all_orient(G, g["cnn"])
    G.relabel()
    _all_orient(G, g["cnn"])
    assert np.array_equal(G.count(policy="bitmap", bias=0, orient=True) + 2, g["cnn"])


def test_orient_rmat16_scan_parity(tmp_path):
    p = accx.rmat_params(16, 16, seed=1)
    G = accx.Graph.generate(p)
    off, dst = G.download()
    ref = oracle.scan(off, dst, 0.3, 4, nthreads=8, out_dir=str(tmp_path))
    _all_orient(G, ref["cnn"])
    G.relabel()
    _all_orient(G, ref["cnn"])
    G.count(policy="bitmap", bias=2, orient=True, out=None)
    r = G.scan(0.3, 4)
    assert np.array_equal(r["sim"], ref["sim"])
    assert np.array_equal(r["label"], ref["label"])
    assert np.array_equal(r["cluster"], ref["cluster"])


def test_orient_chung_lu_heavy_head():
    G = accx.Graph.generate(accx.chung_lu_params(200000, 24, 2.1, 20000, seed=7))
    off, dst = G.download()
    ref = oracle.cn_count(off, dst, nthreads=8)
    for pol in POLICIES:
        assert np.array_equal(G.count(policy=pol, bias=2, orient=True), ref), pol
    G.relabel()
    for pol in POLICIES:
        assert np.array_equal(G.count(policy=pol, bias=2, orient=True), ref), pol


def test_orient_rmat20_equals_direct():
    """R-MAT scale 20: oriented counts equal direct counts entry for entry."""
    G = accx.Graph.generate(accx.rmat_params(20, 16, seed=1))
    G.relabel()
    base = G.count(policy="bitmap")
    for pol in ["bitmap", "heuristic", "merge", "gallop"]:
        c = G.count(policy=pol, orient=True)
        assert np.array_equal(c, base), pol
    assert np.array_equal(G.count(policy="bitmap", orient=True, window_kb=8, sparse_kb=2, block_warps=16), base)


def test_orient_rejects_model_policy():
    G = accx.Graph.generate(accx.rmat_params(10, 8, seed=1))
    with pytest.raises(accx.AccxError):
        G.count(policy="model", orient=True)


def _np_oriented_stats(off, dst):
    """Oriented bucket statistics restated in numpy: owner = longer prefix (ties:
    smaller id), edges whose shorter prefix is empty left out."""
    n = len(off) - 1
    deg = np.diff(off).astype(np.int64)
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    d64 = dst.astype(np.int64)
    pre = np.bincount(src[d64 < src], minlength=n).astype(np.int64)
    pu, pv = pre[src], pre[d64]
    own = (pv > 0) & ((pu > pv) | ((pu == pv) & (src < d64)))
    b = lambda x: np.minimum(np.floor(np.log2(np.maximum(x, 1))).astype(np.int64), 23)
    idx = b(pu[own]) * 24 + b(pv[own])
    e = np.bincount(idx, minlength=576)
    so = np.bincount(idx, weights=pu[own].astype(np.float64), minlength=576)
    sp = np.bincount(idx, weights=pv[own].astype(np.float64), minlength=576)
    return e, so, sp


def test_oriented_bucket_stats_match_numpy():
    G = accx.Graph.generate(accx.chung_lu_params(50000, 16, 2.2, 3000, seed=4))
    off, dst = G.download()
    e, so, sp = G.bucket_stats(orient=True)
    re, rso, rsp = _np_oriented_stats(off, dst)
    assert np.array_equal(e.astype(np.int64), re)
    assert np.array_equal(so, rso) and np.array_equal(sp, rsp)


def _np_direct_stats(off, dst):
    """Direct bucket statistics restated in numpy: owner = larger degree (ties:
    smaller id)."""
    n = len(off) - 1
    deg = np.diff(off).astype(np.int64)
    src = np.repeat(np.arange(n, dtype=np.int64), deg)
    d64 = dst.astype(np.int64)
    du, dv = deg[src], deg[d64]
    own = (du > dv) | ((du == dv) & (src < d64))
    b = lambda x: np.minimum(np.floor(np.log2(np.maximum(x, 1))).astype(np.int64), 23)
    idx = b(du[own]) * 24 + b(dv[own])
    return (np.bincount(idx, minlength=576), np.bincount(idx, weights=du[own].astype(np.float64), minlength=576),
            np.bincount(idx, weights=dv[own].astype(np.float64), minlength=576))


def test_bucket_stats_of_both_modes_after_relabel():
    """Both modes' statistics come from one pass over the relabeled CSR: the
    direct ones equal the original CSR's (degree buckets do not depend on the
    numbering), the oriented ones are those of the relabeled CSR."""
    G = accx.Graph.generate(accx.rmat_params(15, 16, seed=12))
    off, dst = G.download()
    G.relabel()
    roff, rdst, _, _ = G.relabeled_csr()
    for got, ref in ((G.bucket_stats(orient=False), _np_direct_stats(off, dst)),
                     (G.bucket_stats(orient=True), _np_oriented_stats(roff, rdst))):
        assert np.array_equal(got[0].astype(np.int64), ref[0])
        assert np.array_equal(got[1], ref[1]) and np.array_equal(got[2], ref[2])
    G.free()


def test_oriented_model_table_is_argmin_and_counts_are_exact():
    from oracle import mlp_oracle
    m = accx.Model(seed=7)
    G = accx.Graph.generate(accx.rmat_params(15, 16, seed=21))
    ref = G.count(policy="heuristic")
    G.relabel()
    edges, _, _ = G.bucket_stats(orient=True)
    t = m.table_for(G, orient=True).reshape(-1)
    y_ref, _ = mlp_oracle.forward(m.params(), G.bucket_features(orient=True))
    nz = edges > 0
    assert nz.any()
    assert np.array_equal(t[nz], np.argmin(y_ref, 1)[nz])
    with pytest.raises(accx.AccxError):  # no oriented model attached yet
        G.count(policy="model", orient=True)
    G.set_model(m, orient=True)
    assert np.array_equal(G.count(policy="model", orient=True), ref)


def test_kind_bias_steers_the_table():
    m = accx.Model(seed=8)
    G = accx.Graph.generate(accx.rmat_params(14, 16, seed=5))
    ref = G.count(policy="heuristic")
    G.relabel()
    e, _, _ = G.bucket_stats(orient=True)
    m.set_kind_bias([0.0, 0.0, -64.0])
    assert np.allclose(m.kind_bias(), [0, 0, -64])
    t = m.table_for(G, orient=True).reshape(-1)
    assert (t[e > 0] == accx.KIND_BITMAP).all()
    m.set_kind_bias([0.0, -64.0, 0.0])
    t = m.table_for(G, orient=True).reshape(-1)
    assert (t[e > 0] == accx.KIND_GALLOP).all()
    G.set_model(m, orient=True)
    assert np.array_equal(G.count(policy="model", orient=True), ref)
    with pytest.raises(accx.AccxError):
        m.set_kind_bias([0.0, float("nan"), 0.0])
