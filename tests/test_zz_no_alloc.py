"""The allocation-free count (accx_cn_count_noalloc), for callers that cannot
call cudaMalloc, against the regular accx_cn_count through the C ABI.  Three
calls in a row on two different graphs, so a stale scratch list from the
previous call would show.  Collected last on purpose (see the file name)."""
import numpy as np
import pytest

from conftest import has_gpu

pytestmark = pytest.mark.gpu


def test_noalloc_matches_regular_count_on_consecutive_calls():
    import torch
    from acctricnt_gb300 import accx
    graphs = [accx.Graph.generate(accx.rmat_params(14, 16, seed=3)),
              accx.Graph.generate(accx.chung_lu_params(30000, 12, 2.1, 3000, seed=4))]
    refs = [G.count(policy="bitmap", bias=2) for G in graphs]
    for G, ref in [(graphs[0], refs[0]), (graphs[1], refs[1]), (graphs[0], refs[0])]:
        assert 0 < G.m <= accx.cn_count_noalloc_max_entries()
        off_p, dst_p, _ = G.device_ptrs()
        out = torch.full((G.m,), -7, dtype=torch.int32, device="cuda")
        accx.cn_count_noalloc(off_p, dst_p, G.n, G.m, 2, out.data_ptr())
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    import torch
    from acctricnt_gb300 import accx
    G = accx.Graph.generate(accx.rmat_params(8, 4, seed=1))
    off_p, dst_p, _ = G.device_ptrs()
    out = torch.zeros(16, dtype=torch.int32, device="cuda")
    with pytest.raises(accx.AccxError) as ei:
        accx.cn_count_noalloc(off_p, dst_p, G.n, accx.cn_count_noalloc_max_entries() + 2, 0, out.data_ptr())
    assert ei.value.status == accx.ERR_TOO_LARGE
