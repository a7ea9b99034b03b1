"""GPU parity: the sm_103a kernels behind the C ABI against the reference's own
outputs (golden fixtures) and against the oracle on larger seeded graphs.
Counts, similarity bits, labels, clusters and result files must match bit for
bit, for every counting policy and for bitmap windows small enough to force
many windows."""
import os

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


@pytest.mark.parametrize("name", golden_cases())
def test_counts_match_reference_all_policies(name):
    g = load_golden(name)
    G = accx.Graph.from_csr(g["off"], g["dst"])
    for pol in POLICIES:
        cnt = G.count(policy=pol, bias=2)
        assert np.array_equal(cnt, g["cnn"]), pol
    cnt = G.count(policy="table", table=_table(1), bias=2)
    assert np.array_equal(cnt, g["cnn"])
    # tiny shared tables: an 8192-id dense window and a 128-slot sparse table
    # (chunks of 64 ids), so owners are cut into many chunks
    cnt = G.count(policy="bitmap", bias=2, window_kb=1, sparse_kb=1, block_warps=4)
    assert np.array_equal(cnt, g["cnn"])
    G.relabel()
    assert G.relabeled
    for pol in POLICIES:
        assert np.array_equal(G.count(policy=pol, bias=2), g["cnn"]), pol
    cnt = G.count(policy="bitmap", bias=2, window_kb=1, sparse_kb=1, block_warps=8)
    assert np.array_equal(cnt, g["cnn"])
    raw = G.count(policy="heuristic", bias=0)
    assert np.array_equal(raw + 2, g["cnn"])


@pytest.mark.parametrize("name", golden_cases())
def test_scan_matches_reference(name, tmp_path):
    g = load_golden(name)
    G = accx.Graph.from_csr(g["off"], g["dst"])
    G.count(policy="heuristic", bias=0, out=None)
    r = G.scan(float(g["eps"]), int(g["mu"]))
    assert np.array_equal(r["sim"], g["sim"])
    assert np.array_equal(r["label"], g["label"])
    assert np.array_equal(r["cluster"], g["cluster"])
    s = r["summary"]
    assert s["cores"] == int((g["label"] == 1).sum())
    assert s["hubs"] == int((g["label"] == 2).sum())
    assert s["outliers"] == int((g["label"] == 0).sum())
    G.write_result(str(tmp_path), float(g["eps"]), int(g["mu"]))
    with open(os.path.join(str(tmp_path), str(g["result_name"])), "rb") as f:
        assert f.read() == g["result"].tobytes()


@pytest.mark.parametrize("params", [
    ("rmat", 12, 16, 1), ("rmat", 14, 8, 2), ("er", 5000, 20, 3), ("cl", 20000, 16, 4)])
def test_device_generator_matches_host(params):
    kind = params[0]
    if kind == "rmat":
        p = accx.rmat_params(params[1], params[2], seed=params[3])
    elif kind == "er":
        p = accx.er_params(params[1], params[2], seed=params[3])
    else:
        p = accx.chung_lu_params(params[1], params[2], 2.1, 3000, seed=params[3])
    off_h, dst_h = accx.generate_host(p)
    G = accx.Graph.generate(p)
    off_d, dst_d = G.download()
    assert np.array_equal(off_h, off_d) and np.array_equal(dst_h, dst_d)


@pytest.mark.parametrize("eps,mu", [(0.2, 5), (0.5, 5), (0.8, 5)])
def test_rmat16_full_parity_with_oracle(eps, mu, tmp_path):
    """R-MAT scale 16, edge factor 16 (65,536 vertices): the plain CPU config."""
    p = accx.rmat_params(16, 16, seed=1)
    G = accx.Graph.generate(p)
    off, dst = G.download()
    ref = oracle.scan(off, dst, eps, mu, nthreads=8, out_dir=str(tmp_path))
    for pol in POLICIES:
        assert np.array_equal(G.count(policy=pol, bias=2), ref["cnn"]), pol
    G.relabel()
    assert np.array_equal(G.count(policy="bitmap", bias=2), ref["cnn"])
    assert np.array_equal(G.count(policy="bitmap", bias=2, window_kb=2, sparse_kb=2), ref["cnn"])
    r = G.scan(eps, mu)
    assert np.array_equal(r["sim"], ref["sim"])
    assert np.array_equal(r["label"], ref["label"])
    assert np.array_equal(r["cluster"], ref["cluster"])
    assert np.array_equal(G.pairs(), ref["pairs"])
    name = "scanxp-result-%s-%d.txt" % (oracle.eps_string(eps), mu)
    os.rename(os.path.join(str(tmp_path), name), os.path.join(str(tmp_path), "oracle.txt"))
    G.write_result(str(tmp_path), eps, mu)
    with open(os.path.join(str(tmp_path), name), "rb") as a, open(os.path.join(str(tmp_path), "oracle.txt"), "rb") as b:
        assert a.read() == b.read()


def test_chung_lu_skew_parity_with_oracle():
    """Power-law graph with a heavy head: every policy equals the oracle."""
    p = accx.chung_lu_params(200000, 24, 2.1, 20000, seed=7)
    G = accx.Graph.generate(p)
    off, dst = G.download()
    ref = oracle.cn_count(off, dst, nthreads=8)
    for pol in POLICIES:
        assert np.array_equal(G.count(policy=pol, bias=2), ref), pol
    G.relabel()
    for pol in POLICIES:
        assert np.array_equal(G.count(policy=pol, bias=2), ref), pol


@pytest.mark.parametrize("kind", ["chung_lu", "erdos_renyi"])
def test_skew_config_scaled_down_parity_with_oracle(kind, default_sched):
    """The learned-scheduler skew config scaled down by 10: Chung-Lu with 2M
    vertices, exponent 2.1, mean degree 24, max expected degree 100K (the
    20M-vertex config's max-degree/n ratio), and Erdos-Renyi with 2M vertices,
    mean degree 24.  The scheduler's plan and every fixed policy in both modes
    equal the oracle's CheckCoreBitmap entry for entry."""
    if kind == "chung_lu":
        p = accx.chung_lu_params(2_000_000, 24, 2.1, 1e5, seed=1)
    else:
        p = accx.er_params(2_000_000, 24, seed=1)
    G = accx.Graph.generate(p)
    off, dst = G.download()
    ref = oracle.cn_count(off, dst, nthreads=0)
    assert np.array_equal(G.count(policy="heuristic", bias=2), ref)
    G.relabel()
    pl = default_sched.plan(G)
    assert np.array_equal(G.count(policy="model", orient=pl["orient"], bias=2), ref)
    for pol in ("gallop", "bitmap"):
        assert np.array_equal(G.count(policy=pol, bias=2), ref), pol
    for pol in ("merge", "gallop", "bitmap"):
        assert np.array_equal(G.count(policy=pol, bias=2, orient=True), ref), pol
    if kind == "chung_lu":
        assert np.diff(off.astype(np.int64)).max() > 20_000  # the heavy head is there


@pytest.mark.parametrize("kind", ["chung_lu", "erdos_renyi"])
def test_skew_config_full_size_parity_with_oracle(kind, default_sched):
    """The learned-scheduler skew config at full size: Chung-Lu with 20M vertices,
    exponent 2.1, mean degree 24, max expected degree 1M (444.9M entries), and
    Erdos-Renyi with 20M vertices, mean degree 24 (480.0M entries).  The
    scheduler's tuned plan (as the bench runs it) and the reference's ratio-50
    rule equal the oracle's CheckCoreBitmap (all host threads) entry for entry."""
    from acctricnt_gb300 import workloads
    p = workloads.chung_lu_20m() if kind == "chung_lu" else workloads.er_20m()
    G = accx.Graph.generate(p)
    off, dst = G.download()
    ref = oracle.cn_count(off, dst, nthreads=0)
    assert np.array_equal(G.count(policy="heuristic", bias=2), ref)
    G.relabel()
    pl = default_sched.plan(G, tune=True)
    assert np.array_equal(G.count(policy="model", orient=pl["orient"], bias=2), ref)
    G.free()


def test_large_rmat_policies_agree_and_are_symmetric():
    """Size-independent properties at R-MAT scale 20: all policies agree, the
    count array is symmetric (cnt[e] == cnt[reverse(e)]), and sampled entries
    equal an independent numpy set intersection."""
    G = accx.Graph.generate(accx.rmat_params(20, 16, seed=1))
    off, dst = G.download()
    base = G.count(policy="heuristic")
    for pol in ["merge", "bitmap", "gallop"]:
        assert np.array_equal(G.count(policy=pol), base), pol
    G.relabel()
    assert np.array_equal(G.count(policy="bitmap"), base)
    assert np.array_equal(G.count(policy="bitmap", window_kb=16, sparse_kb=4), base)
    n = len(off) - 1
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(off).astype(np.int64))
    key = src * n + dst
    rkey = dst.astype(np.int64) * n + src
    order = np.argsort(key)
    pos = order[np.searchsorted(key[order], rkey)]
    assert np.array_equal(base[pos], base)
    rng = np.random.default_rng(0)
    for e in rng.integers(0, len(dst), 2000):
        u, v = src[e], dst[e]
        a = dst[off[u]:off[u + 1]]
        b = dst[off[v]:off[v + 1]]
        assert base[e] == len(np.intersect1d(a, b, assume_unique=True))


def test_plain_cpu_config_matches_reference_digests(tmp_path):
    """R-MAT scale 16, edge factor 16, seed 1, eps 0.2, mu 5 (the plain CPU
    config): every GPU output has the sha256 digest of the reference build's own
    output (tests/golden/rmat16_e02_mu5_digests.json, from oracle/_ref/ref_harness),
    for direct and oriented counts, relabeled or not."""
    import hashlib
    import json
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "rmat16_e02_mu5_digests.json")) as f:
        fx = json.load(f)
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    G = accx.Graph.generate(accx.rmat_params(16, 16, seed=1))
    off, dst = G.download()
    assert sha(off) == fx["graph_sha256"]["off"] and sha(dst) == fx["graph_sha256"]["dst"]
    for kw in (dict(policy="heuristic"), dict(policy="bitmap"), dict(policy="bitmap", orient=True)):
        assert sha(G.count(bias=2, **kw)) == fx["sha256"]["cnn"], kw
    G.relabel()
    for kw in (dict(policy="merge"), dict(policy="bitmap", orient=True), dict(policy="gallop", orient=True)):
        assert sha(G.count(bias=2, **kw)) == fx["sha256"]["cnn"], kw
    r = G.scan(fx["eps"], fx["mu"])
    for k in ("sim", "label", "cluster"):
        assert sha(r[k]) == fx["sha256"][k], k
    G.write_result(str(tmp_path), fx["eps"], fx["mu"])
    with open(os.path.join(str(tmp_path), fx["result_name"]), "rb") as f:
        assert hashlib.sha256(f.read()).hexdigest() == fx["result_sha256"]


def test_rmat24_full_parity_with_oracle():
    """The bench workload at full size, R-MAT scale 24 (16.8M vertices, 520.8M
    entries): all counts of the oriented count on the relabeled copy (the bench's
    plan) and of the reference's ratio-50 heuristic equal the oracle's
    CheckCoreBitmap (all host threads) entry for entry, and the SCAN query's
    similarity bits, labels, clusters and non-core pairs equal the oracle's at
    eps 0.2, 0.5 and 0.8, mu 5.  Also: the triangle total is an integer equal to
    accx_triangles, and 4096 sampled entries are symmetric and equal numpy set
    intersections on the caller's CSR."""
    G = accx.Graph.generate(accx.rmat_params(24, 16, seed=1))
    off, dst = G.download()
    ref = oracle.cn_count(off, dst, nthreads=0)
    assert np.array_equal(G.count(policy="heuristic", bias=2), ref)
    G.relabel()
    assert np.array_equal(G.count(policy="bitmap", bias=2, orient=True), ref)
    for eps in (0.2, 0.5, 0.8):
        want = oracle.scan_from_counts(off, dst, ref, eps, 5, nthreads=0)
        r = G.scan(eps, 5)
        assert np.array_equal(r["sim"], want["sim"]), eps
        assert np.array_equal(r["label"], want["label"]), eps
        assert np.array_equal(r["cluster"], want["cluster"]), eps
        assert np.array_equal(G.pairs(), want["pairs"]), eps
        del want, r
    direct = ref
    s = int(direct.sum(dtype=np.int64)) - 2 * len(dst)
    assert s % 6 == 0 and G.triangles() == s // 6
    rng = np.random.default_rng(24)
    for e in rng.integers(0, len(dst), 4096):
        u = int(np.searchsorted(off, e, side="right")) - 1
        v = int(dst[e])
        a = dst[off[u]:off[u + 1]]
        b = dst[off[v]:off[v + 1]]
        r = int(off[v]) + int(np.searchsorted(b, u))
        assert dst[r] == u and direct[r] == direct[e]
        assert direct[e] == 2 + len(np.intersect1d(a, b, assume_unique=True))
    G.free()


@pytest.mark.parametrize("mode", [True, "exact"])
@pytest.mark.parametrize("bad", ["self_loop", "unsorted", "asymmetric", "range"])
def test_invalid_graphs_rejected(bad, mode):
    off = np.array([0, 2, 4, 6], np.uint32)
    dst = np.array([1, 2, 0, 2, 0, 1], np.int32)
    code = {"self_loop": accx.ERR_SELF_LOOP, "unsorted": accx.ERR_UNSORTED, "asymmetric": accx.ERR_ASYMMETRIC,
            "range": accx.ERR_RANGE}[bad]
    if bad == "self_loop":
        dst = np.array([0, 2, 0, 2, 0, 1], np.int32)
    elif bad == "unsorted":
        dst = np.array([2, 1, 0, 2, 0, 1], np.int32)
    elif bad == "asymmetric":
        off = np.array([0, 2, 3, 5], np.uint32)
        dst = np.array([1, 2, 0, 0, 1], np.int32)
    else:
        dst = np.array([1, 9, 0, 2, 0, 1], np.int32)
    with pytest.raises(accx.AccxError) as ei:
        accx.Graph.from_csr(off, dst, validate=mode)
    assert ei.value.status == code


@pytest.mark.parametrize("mode", [True, "exact"])
@pytest.mark.parametrize("case", ["directed_cycle", "swapped_targets", "one_edge_moved"])
def test_asymmetric_graphs_with_balanced_degrees_rejected(case, mode):
    """Every vertex is a neighbour as often as its own list is long, yet the
    graph is not symmetric: in the exact check the row-of-neighbour test of the
    sorted entries (not the degree test) has to catch these; the fingerprints
    catch them too."""
    if case == "directed_cycle":
        off, dst = np.array([0, 1, 2, 3], np.uint32), np.array([1, 2, 0], np.int32)
    elif case == "swapped_targets":  # the edges 0-1 and 2-3 with one target of each pair swapped
        off, dst = np.array([0, 1, 2, 3, 4], np.uint32), np.array([3, 0, 1, 2], np.int32)
    else:  # a large symmetric graph with one entry's target moved (rows stay sorted)
        off, dst = accx.generate_host(accx.rmat_params(16, 16, seed=3))
        dst = dst.copy()
        deg = np.diff(off.astype(np.int64))
        u = int(np.nonzero(deg >= 3)[0][len(np.nonzero(deg >= 3)[0]) // 2])
        row = dst[off[u]:off[u + 1]]
        lo, hi = int(row[0]), int(row[1])
        assert hi - lo >= 1
        w = next((x for x in range(lo + 1, hi) if x != u), None)
        if w is None:  # the first gap of the row between two consecutive targets
            i = next(i for i in range(len(row) - 1) if row[i + 1] - row[i] > 1 and row[i] + 1 != u)
            dst[off[u] + i] = row[i] + 1
        else:
            dst[off[u]] = w
    with pytest.raises(accx.AccxError) as ei:
        accx.Graph.from_csr(off, dst, validate=mode)
    assert ei.value.status == accx.ERR_ASYMMETRIC


@pytest.mark.parametrize("validate", [True, "exact", False])
def test_reverse_index_sources_give_the_same_counts(validate):
    """The oriented count's reverse index comes from exact validation (original
    CSR), from the sort (a known-symmetric handle: validated or generated) or
    from the search (an unvalidated handle): the same counts."""
    off, dst = accx.generate_host(accx.rmat_params(14, 16, seed=8))
    ref = oracle.cn_count(off, dst, 2)
    G = accx.Graph.from_csr(off, dst, validate=validate)
    assert np.array_equal(G.count(policy="bitmap", bias=2, orient=True), ref)
    G.relabel()
    assert np.array_equal(G.count(policy="bitmap", bias=2, orient=True), ref)
    G.free()


@pytest.mark.parametrize("shift", [0, 1])
def test_counts_into_pinned_host_memory(shift):
    """A count into pinned host memory: written by the relabeled count's final
    gather when the buffer is 16-byte aligned (shift 0), through the copy
    otherwise (shift 1 entry); the same counts as into pageable memory, and the
    resident counts stay valid for queries."""
    torch = pytest.importorskip("torch")
    off, dst = accx.generate_host(accx.rmat_params(15, 16, seed=9))
    ref = oracle.cn_count(off, dst, 2)
    G = accx.Graph.from_csr(off, dst)
    G.relabel()
    buf = torch.full((len(dst) + 4,), -7, dtype=torch.int32).pin_memory()
    for orient in (True, False):
        buf.fill_(-7)
        G.count(policy="bitmap", bias=2, out=buf.data_ptr() + 4 * shift, orient=orient)
        got = buf.numpy()
        assert np.array_equal(got[shift:shift + len(dst)], ref), orient
        assert np.all(got[:shift] == -7) and np.all(got[shift + len(dst):] == -7)
        assert np.array_equal(G.read_counts(), ref)
    G.free()


def test_query_before_count_is_not_ready():
    off, dst = accx.generate_host(accx.rmat_params(8, 8))
    G = accx.Graph.from_csr(off, dst)
    with pytest.raises(accx.AccxError) as ei:
        G.scan(0.5, 2)
    assert ei.value.status == accx.ERR_NOT_READY
