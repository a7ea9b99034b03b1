"""The C ABI library loads and exports every function include/accx.h declares;
host-only entry points behave without a GPU."""
import os
import re

import numpy as np
import pytest

from acctricnt_gb300 import accx
from conftest import ROOT, has_gpu
from oracle import oracle


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "accx.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(accx_\w+)\s*\(", txt)))


def test_exports_every_declared_symbol():
    names = declared_functions()
    assert len(names) >= 19
    missing = [n for n in names if not hasattr(accx.lib, n)]
    assert not missing, missing


def test_version_and_strerror():
    assert "sm_103a" in accx.version()
    for code in range(0, -14, -1):
        assert accx.strerror(code)
    assert accx.strerror(accx.ERR_SELF_LOOP) == "Self loop"


@pytest.mark.parametrize("eps", [0.2, 0.5, 0.8, 1.0, 0.0, 0.123456, 0.1000001, 12.5, 0.30000000000000004])
def test_eps_string_matches_reference_rule(eps):
    assert accx.eps_string(eps) == oracle.eps_string(eps)


def test_host_generator_is_deterministic():
    a = accx.generate_host(accx.rmat_params(9, 8, seed=5))
    b = accx.generate_host(accx.rmat_params(9, 8, seed=5))
    c = accx.generate_host(accx.rmat_params(9, 8, seed=6))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[1][:100], c[1][:100]) or len(a[1]) != len(c[1])
    for off, dst in (a, accx.generate_host(accx.er_params(500, 6)),
                     accx.generate_host(accx.chung_lu_params(800, 8, 2.1, 200))):
        assert oracle.check_graph(off, dst) == 0
        # symmetric
        n = len(off) - 1
        src = np.repeat(np.arange(n), np.diff(off))
        fwd = set(zip(src.tolist(), dst.tolist()))
        assert all((v, u) in fwd for u, v in fwd)


def test_chung_lu_has_a_heavy_head():
    off, dst = accx.generate_host(accx.chung_lu_params(20000, 24, 2.1, 5000, seed=1))
    deg = np.diff(off)
    assert deg.max() > 2000 and abs(deg.mean() - 24) < 6


def test_graph_files_roundtrip(tmp_path):
    off, dst = accx.generate_host(accx.rmat_params(8, 8))
    accx.write_graph_dir(str(tmp_path), off, dst)
    hdr = np.fromfile(str(tmp_path / "b_degree.bin"), np.uint32)
    assert hdr[0] == 4 and hdr[1] == len(off) - 1 and hdr[2] == len(dst)
    assert np.array_equal(hdr[3:].astype(np.int64), np.diff(off).astype(np.int64))
    assert np.array_equal(np.fromfile(str(tmp_path / "b_adj.bin"), np.int32), dst)


def test_invalid_arguments_return_status():
    with pytest.raises(accx.AccxError) as ei:
        accx.generate_host(accx.gen_params(7, 1, 1))
    assert ei.value.status == accx.ERR_INVALID_ARG


@pytest.mark.skipif(has_gpu(), reason="checks the no-device status")
def test_no_device_status():
    off, dst = accx.generate_host(accx.rmat_params(6, 4))
    with pytest.raises(accx.AccxError) as ei:
        accx.Graph.from_csr(off, dst)
    assert ei.value.status in (accx.ERR_NO_DEVICE, accx.ERR_CUDA)


def test_scheduler_rejects_too_many_candidates():
    """Checked before any device work."""
    with pytest.raises(accx.AccxError) as ei:
        accx.Scheduler.train(candidates=accx.SCHED_MAX_CANDIDATES + 1)
    assert ei.value.status == accx.ERR_INVALID_ARG


def _sched_text(version, with_candidates):
    model = "0 " * accx.MODEL_NPARAMS
    info = "info 100 10 1 -1 1 1 1 0 " + "1 " * accx.SCHED_NOFFSETS
    if with_candidates:
        info += "3 1 " + "1 " * accx.SCHED_MAX_CANDIDATES
    body = "".join("model %d 0 0 -1\n%s\n%s\n" % (o, model, info) for o in (0, 1))
    return "accx-sched %d\n%s" % (version, body)


@pytest.mark.parametrize("text", [_sched_text(3, True), _sched_text(2, False), "accx-sched 2\nmodel 1 0 0 0\n",
                                  "not a scheduler file\n"])
def test_malformed_scheduler_files_are_rejected(tmp_path, text):
    """Unknown versions, a version-2 file without its candidates record, models
    out of order and foreign files: an I/O status, found while parsing (before
    any model reaches the device)."""
    p = tmp_path / "bad.model"
    p.write_text(text)
    with pytest.raises(accx.AccxError) as ei:
        accx.Scheduler.load(str(p))
    assert ei.value.status == accx.ERR_IO
