"""The SCAN_XP drop-in CLIs (main_scanxp / experimental main_scanxp argument
layouts): result files byte-identical to the reference's on the golden graphs."""
import os
import subprocess

import numpy as np
import pytest

from acctricnt_gb300 import BUILD_DIR, accx
from conftest import golden_cases, load_golden

CLI = os.path.join(BUILD_DIR, "scan-xp-gb300")
CLI_VAR = os.path.join(BUILD_DIR, "scan-xp-gb300-varying")


def test_cli_usage_and_missing_graph(tmp_path):
    r = subprocess.run([CLI], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage" in r.stdout
    r = subprocess.run([CLI, str(tmp_path / "nope"), "0.2", "5", "1"], capture_output=True, text=True)
    assert r.returncode == 1 and "cannot be read" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_cases())
@pytest.mark.parametrize("variant", ["model", "fallback", "varying", "heuristic_norelabel", "oriented_bitmap"])
def test_cli_result_file_matches_reference(name, variant, tmp_path, quick_sched_file):
    """With a scheduler file (the learned plan) and without one (the reference's
    ratio-50 rule), and under explicit policies: the same result file, byte for
    byte the reference's."""
    g = load_golden(name)
    d = str(tmp_path)
    accx.write_graph_dir(d, g["off"], g["dst"])
    eps, mu = repr(float(g["eps"])), str(int(g["mu"]))
    env = dict(os.environ, ACCX_SCHED_MODEL=quick_sched_file)
    if variant == "varying":
        cmd = [CLI_VAR, d, eps, mu, "4", "1", "8", os.path.join(d, "log.txt")]
    else:
        cmd = [CLI, d, eps, mu, "4", os.path.join(d, "log.txt")]
    if variant == "fallback":
        env.update(ACCX_SCHED_MODEL=os.path.join(d, "no-such.model"))
    if variant == "heuristic_norelabel":
        env.update(ACCX_POLICY="heuristic", ACCX_RELABEL="0")
    if variant == "oriented_bitmap":
        env.update(ACCX_POLICY="bitmap", ACCX_ORIENT="1")
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    with open(os.path.join(d, str(g["result_name"])), "rb") as f:
        assert f.read() == g["result"].tobytes()
    log = open(os.path.join(d, "log.txt")).read()
    assert "Step1 - CheckCore" in log
    if variant in ("model", "varying"):
        assert "kernel plan: learned scheduler" in log
    if variant == "fallback":
        assert "kernel plan: reference ratio-50 rule" in log


def _np_convert(text):
    """The reference converter's rules restated: '#' lines skipped, pairs with
    first < second kept, n = largest kept id + 1, both directions, rows sorted."""
    pairs = set()
    mx = -1
    for line in text.decode().split("\n"):
        if not line or line[0] == "#":
            continue
        parts = line.split()
        if len(parts) < 2:
            continue
        a, b = int(parts[0]), int(parts[1])
        if a < b:
            pairs.add((a, b))
            mx = max(mx, b)
    n = mx + 1
    rows = [[] for _ in range(n)]
    for a, b in pairs:
        rows[a].append(b)
        rows[b].append(a)
    deg = np.array([len(r) for r in rows], np.int32)
    adj = np.array([v for r in rows for v in sorted(r)], np.int32)
    head = np.array([4, n, len(adj)], np.uint32).view(np.int32)
    return np.concatenate([head, deg]).tobytes(), adj.tobytes()


def test_edge_list_fixture_matches_the_restated_rules():
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "edge_list_converter.npz"))
    deg, adj = _np_convert(g["edges_txt"].tobytes())
    assert deg == g["b_degree_bin"].tobytes() and adj == g["b_adj_bin"].tobytes()


@pytest.mark.gpu
def test_edge_list_converter_matches_reference(tmp_path):
    conv = os.path.join(os.path.dirname(CLI), "edge-list-to-bins-gb300")
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "edge_list_converter.npz"))
    src = tmp_path / "edges.txt"
    src.write_bytes(g["edges_txt"].tobytes())
    r = subprocess.run([conv, str(src), str(tmp_path / "d.bin"), str(tmp_path / "a.bin")], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    assert (tmp_path / "d.bin").read_bytes() == g["b_degree_bin"].tobytes()
    assert (tmp_path / "a.bin").read_bytes() == g["b_adj_bin"].tobytes()
    # a repeated edge: degrees count it once, as the adjacency does; the result loads and counts
    src.write_bytes(b"0 1\n0 1\n1 2\n0 2\n2 3")
    r = subprocess.run([conv, str(src), str(tmp_path / "b_degree.bin"), str(tmp_path / "b_adj.bin")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    deg, adj = _np_convert(b"0 1\n1 2\n0 2\n2 3\n")
    assert (tmp_path / "b_degree.bin").read_bytes() == deg and (tmp_path / "b_adj.bin").read_bytes() == adj
    G = accx.Graph.load_dir(str(tmp_path))
    assert G.count(policy="bitmap", bias=2, orient=True).tolist() == [3, 3, 3, 3, 3, 3, 2, 2]
    # empty input
    src.write_bytes(b"# nothing\n")
    r = subprocess.run([conv, str(src), str(tmp_path / "d0.bin"), str(tmp_path / "a0.bin")], capture_output=True)
    assert r.returncode == 0 and (tmp_path / "a0.bin").read_bytes() == b""
