"""The oriented counting scheme restated on the CPU (no GPU), against the
reference's own counts in the golden fixtures.

For an undirected edge {x, y} the owner is the endpoint with the longer prefix
P(.) = N(.) ∩ [0, .) (ties: the smaller id), the partner the other one.  The
owner's prefix is the probe set; the partner's prefix, cut at min(x, y), is the
probe list.  Every common id z closes the triangle z < min(x, y) < max(x, y),
which is met exactly once, on the edge of its two largest vertices.  A hit adds
one to three prefix entries -- (partner, z), (owner, z) and the edge's own
prefix entry (in the larger endpoint's row) -- and a final pass copies every
prefix entry's count to its reverse.  The count is bias + credits.  This is the
rule set of k_classify / k_bitmap_or / k_combine_or (the GPU kernels), written
out plainly; tests/test_orient.py checks the kernels themselves.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden


def oriented_counts(off, dst, bias=2):
    off = off.astype(np.int64)
    dst = dst.astype(np.int64)
    n = len(off) - 1
    rows = [dst[off[u]:off[u + 1]] for u in range(n)]
    pre = [int(np.searchsorted(r, u)) for u, r in enumerate(rows)]  # rows are sorted
    pos = {}
    for u in range(n):
        for k, v in enumerate(rows[u]):
            pos[(u, int(v))] = int(off[u]) + k
    cnt = np.zeros(len(dst), np.int64)
    for u in range(n):
        for v in rows[u]:
            v = int(v)
            if v > u:
                continue  # each undirected edge once, from its larger endpoint's row
            x, y = u, v
            o, p = (x, y) if (pre[x] > pre[y] or (pre[x] == pre[y] and x < y)) else (y, x)
            probe_set = set(int(z) for z in rows[o][:pre[o]])
            cut = min(x, y)
            for z in rows[p][:pre[p]]:
                z = int(z)
                if z >= cut:
                    break
                if z in probe_set:
                    cnt[pos[(p, z)]] += 1  # partner-side entry
                    cnt[pos[(o, z)]] += 1  # owner-side entry
                    cnt[pos[(max(x, y), min(x, y))]] += 1  # the edge's prefix entry
    # suffix entries take their reverse prefix entry's count
    out = cnt.copy()
    for u in range(n):
        for v in rows[u]:
            v = int(v)
            if v > u:
                out[pos[(u, v)]] = cnt[pos[(v, u)]]
    return out + bias


@pytest.mark.parametrize("name", golden_cases())
def test_oriented_scheme_matches_reference_counts(name):
    g = load_golden(name)
    if len(g["dst"]) > 200000:
        pytest.skip("pure-Python restatement: small fixtures only")
    assert np.array_equal(oriented_counts(g["off"], g["dst"]), g["cnn"].astype(np.int64))


def test_every_triangle_is_met_once():
    # K5: 10 triangles, each edge in 3 of them
    n = 5
    dst = np.array([v for u in range(n) for v in range(n) if v != u], np.int32)
    off = np.arange(0, n * (n - 1) + 1, n - 1, dtype=np.uint32)
    c = oriented_counts(off, dst, bias=0)
    assert np.all(c == 3) and c.sum() // 6 == 10
