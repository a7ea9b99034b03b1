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
@pytest.mark.parametrize("variant", ["plain", "varying", "heuristic_norelabel", "direct"])
def test_cli_result_file_matches_reference(name, variant, tmp_path):
    g = load_golden(name)
    d = str(tmp_path)
    accx.write_graph_dir(d, g["off"], g["dst"])
    eps, mu = repr(float(g["eps"])), str(int(g["mu"]))
    env = dict(os.environ)
    if variant == "varying":
        cmd = [CLI_VAR, d, eps, mu, "4", "1", "8", os.path.join(d, "log.txt")]
    else:
        cmd = [CLI, d, eps, mu, "4", os.path.join(d, "log.txt")]
    if variant == "heuristic_norelabel":
        env.update(ACCX_POLICY="heuristic", ACCX_RELABEL="0")
    if variant == "direct":  # the reference's formulation: full-list intersections
        env.update(ACCX_ORIENT="0")
    r = subprocess.run(cmd, capture_output=True, text=True, env=env)
    assert r.returncode == 0, r.stderr
    with open(os.path.join(d, str(g["result_name"])), "rb") as f:
        assert f.read() == g["result"].tobytes()
    assert "Step1 - CheckCore" in open(os.path.join(d, "log.txt")).read()
