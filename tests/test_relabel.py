"""Degree-descending relabel on the GPU -- the reference's "deg" reorder
(ReorderDegDescending + Reorder, scan-query/scan_xp.cpp:1145-1222, :1279-1301;
maps back through old_vid_dict, scan-query/util/graph.cpp:176-216).

The relabeled CSR and its maps are compared with a numpy restatement on graphs
whose rows fall in every degree class of the row sort (at most 1, 32, 256,
1024 and 4096 entries, and above), including rows exactly at each class bound.
"""
import numpy as np
import pytest

from conftest import golden_cases, has_gpu, load_golden

pytestmark = pytest.mark.gpu


def np_relabel(off, dst):
    """roff, rdst, map (original entry -> new position), oldid (new -> original)."""
    n = len(off) - 1
    deg = np.diff(off.astype(np.int64))
    oldid = np.lexsort((np.arange(n), -deg))  # degree descending, ties by id
    newid = np.empty(n, np.int64)
    newid[oldid] = np.arange(n)
    src = np.repeat(np.arange(n), deg)
    nu, nv = newid[src], newid[dst.astype(np.int64)]
    order = np.lexsort((nv, nu))  # new position -> original entry
    roff = np.zeros(n + 1, np.int64)
    roff[1:] = np.cumsum(deg[oldid])
    rmap = np.empty(len(dst), np.int64)
    rmap[order] = np.arange(len(dst))
    return roff, nv[order], rmap, oldid


def csr_from_edges(n, edges):
    e = np.asarray(edges, np.int64)
    e = np.concatenate([e, e[:, ::-1]])
    e = np.unique(e[e[:, 0] != e[:, 1]], axis=0)
    off = np.zeros(n + 1, np.uint32)
    off[1:] = np.cumsum(np.bincount(e[:, 0], minlength=n))
    return off, e[:, 1].astype(np.int32)


def stars_at_class_bounds(seed=5):
    """Disjoint stars whose centres have degree at and around every class bound,
    tied with a sprinkle of random edges among the leaves."""
    rng = np.random.default_rng(seed)
    edges, nxt = [], 0
    for d in (5000, 4097, 4096, 4095, 1025, 1024, 1023, 257, 256, 255, 33, 32, 31, 2, 1):
        c = nxt
        edges += [(c, c + 1 + i) for i in range(d)]
        nxt = c + 1 + d
    n = nxt + 3  # three isolated vertices
    leaves = rng.integers(0, nxt, size=(3000, 2))
    edges += [tuple(x) for x in leaves]
    return csr_from_edges(n, edges)


def check(G, off, dst):
    G.relabel()
    roff, rdst, rmap, oldid = G.relabeled_csr()
    e_roff, e_rdst, e_rmap, e_oldid = np_relabel(off, dst)
    assert np.array_equal(roff.astype(np.int64), e_roff)
    assert np.array_equal(oldid.astype(np.int64), e_oldid)
    assert np.array_equal(rdst.astype(np.int64), e_rdst)
    assert np.array_equal(rmap.astype(np.int64), e_rmap)


@pytest.mark.skipif(not has_gpu(), reason="needs a GPU")
@pytest.mark.parametrize("name", golden_cases())
def test_relabel_golden(name):
    from acctricnt_gb300 import accx
    g = load_golden(name)
    G = accx.Graph.from_csr(g["off"], g["dst"])
    check(G, g["off"], g["dst"])
    G.free()


@pytest.mark.skipif(not has_gpu(), reason="needs a GPU")
def test_relabel_class_bounds():
    from acctricnt_gb300 import accx
    off, dst = stars_at_class_bounds()
    G = accx.Graph.from_csr(off, dst)
    check(G, off, dst)
    # counts through the relabeled copy equal the direct ones
    base = G.count(policy="merge", bias=2)
    assert np.array_equal(G.count(policy="bitmap", bias=2, orient=True), base)
    G.free()


@pytest.mark.skipif(not has_gpu(), reason="needs a GPU")
@pytest.mark.parametrize("gen", ["rmat18", "chung_lu"])
def test_relabel_generated(gen):
    from acctricnt_gb300 import accx
    p = accx.rmat_params(18, 16, seed=3) if gen == "rmat18" else accx.chung_lu_params(200000, 24, max_degree=20000, seed=4)
    G = accx.Graph.generate(p)
    off, dst = G.download()
    assert np.diff(off.astype(np.int64)).max() > 4096  # rows for the segmented sort too
    check(G, off, dst)
    G.free()
