"""Edge lists to graphs on the device (the converter's job), triangle totals,
count persistence, and the filtered-cost vertex-range partitioner."""
import numpy as np
import pytest

from conftest import golden_cases, has_gpu, load_golden

if has_gpu():
    from acctricnt_gb300 import accx
from oracle import oracle


def _ranges_fixture():
    import json
    import os
    from conftest import GOLDEN
    with open(os.path.join(GOLDEN, "vertex_ranges.json")) as f:
        return json.load(f)


def _ranges_graph(name):
    from acctricnt_gb300 import accx as ax
    if name == "rmat16":
        return ax.generate_host(ax.rmat_params(16, 16, seed=1))
    g = load_golden(name)
    return g["off"], g["dst"]


@pytest.mark.parametrize("name", sorted(_ranges_fixture()["ranges"]))
def test_oracle_vertex_ranges_equal_the_reference_partitioner(name):
    """Ranges recorded from the reference's own
    ComputeVertexRangeAccumulatedFilteredDegree (oracle/_ref/ref_ranges)."""
    fx = _ranges_fixture()
    off, dst = _ranges_graph(name)
    for parts, want in zip(fx["parts"], fx["ranges"][name]):
        assert oracle.vertex_ranges(off, dst, parts).tolist() == want, parts


def test_oracle_vertex_ranges_cover_and_balance():
    from acctricnt_gb300 import accx as ax
    off, dst = ax.generate_host(ax.rmat_params(12, 16, seed=3))
    r = oracle.vertex_ranges(off, dst, 4)
    assert r[0] == 0 and r[-1] == len(off) - 1 and np.all(np.diff(r.astype(np.int64)) >= 0)


@pytest.mark.gpu
def test_from_edges_matches_the_converter_semantics():
    rng = np.random.default_rng(2)
    n = 3000
    src = rng.integers(0, n, 40000).astype(np.uint32)
    dst = rng.integers(0, n, 40000).astype(np.uint32)
    src[:50] = dst[:50]  # self loops
    src = np.concatenate([src, dst[:500]])  # reversed duplicates
    dst = np.concatenate([dst, src[:500]])
    G = accx.Graph.from_edges(src, dst, n)
    off, d = G.download()
    keep = src != dst
    pairs = np.unique(np.concatenate([src[keep].astype(np.int64) * n + dst[keep], dst[keep].astype(np.int64) * n + src[keep]]))
    assert np.array_equal(d, (pairs % n).astype(np.int32))
    assert np.array_equal(np.diff(off), np.bincount(pairs // n, minlength=n))
    with pytest.raises(accx.AccxError) as ei:
        accx.Graph.from_edges(np.array([1], np.uint32), np.array([n], np.uint32), n)
    assert ei.value.status == accx.ERR_RANGE


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_cases())
def test_triangles_and_persistence(name, tmp_path):
    g = load_golden(name)
    G = accx.Graph.from_csr(g["off"], g["dst"])
    G.count(policy="bitmap", bias=2, out=None)
    assert G.triangles() == int((g["cnn"].astype(np.int64) - 2).sum() // 6)
    p = str(tmp_path / "counts.bin")
    G.save_counts(p)
    H = accx.Graph.from_csr(g["off"], g["dst"])
    H.load_counts(p)
    assert np.array_equal(H.read_counts(), g["cnn"])
    r = H.scan(float(g["eps"]), int(g["mu"]))
    assert np.array_equal(r["label"], g["label"]) and np.array_equal(r["cluster"], g["cluster"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(_ranges_fixture()["ranges"]))
def test_vertex_ranges_equal_the_reference_partitioner(name):
    fx = _ranges_fixture()
    off, dst = _ranges_graph(name)
    G = accx.Graph.from_csr(off, dst)
    for parts, want in zip(fx["parts"], fx["ranges"][name]):
        assert G.vertex_ranges(parts).tolist() == want, parts


@pytest.mark.gpu
@pytest.mark.parametrize("parts", [1, 2, 3, 8])
def test_vertex_ranges_equal_the_oracle(parts):
    G = accx.Graph.generate(accx.rmat_params(16, 16, seed=5))
    off, dst = G.download()
    assert np.array_equal(G.vertex_ranges(parts), oracle.vertex_ranges(off, dst, parts))


@pytest.mark.gpu
def test_pinned_host_buffers_roundtrip():
    """Graph upload and count download through pinned (GPU-mapped) host buffers
    -- the copy-kernel path -- equal the pageable path, for sizes that are not
    multiples of 16 bytes and for a buffer that starts 4 bytes into its block."""
    import ctypes
    import torch
    off, dst = accx.generate_host(accx.rmat_params(13, 7, seed=21))
    n, m = len(off) - 1, len(dst)
    ref = accx.Graph.from_csr(off, dst).count(policy="bitmap", bias=2)
    for shift in (0, 1):
        t_off = torch.zeros(n + 1 + shift, dtype=torch.int32).pin_memory()
        t_dst = torch.zeros(m + shift, dtype=torch.int32).pin_memory()
        t_off[shift:] = torch.from_numpy(off.view(np.int32))
        t_dst[shift:] = torch.from_numpy(dst)
        H = accx.Graph.from_device(t_off.data_ptr() + 4 * shift, t_dst.data_ptr() + 4 * shift, n, m, validate=True)
        o2, d2 = H.download()
        assert np.array_equal(o2, off) and np.array_equal(d2, dst)
        out = torch.full((m + shift,), -7, dtype=torch.int32).pin_memory()
        H.count(policy="bitmap", bias=2, orient=True, out=None)
        accx._check(accx.lib.accx_cn_read(H._h, ctypes.c_void_p(out.data_ptr() + 4 * shift), None), "cn_read")
        assert np.array_equal(out[shift:].numpy(), ref)
        H.free()
