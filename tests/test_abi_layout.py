"""The ctypes mirrors of the C ABI's structs (acctricnt_gb300/accx.py) have the
layout include/accx.h gives them: a C program built with the host compiler
prints every struct's size and every field's offset, and the two must agree
(a field added on one side only would shift every later field)."""
import ctypes
import os
import shutil
import subprocess

import pytest

from acctricnt_gb300 import accx
from conftest import ROOT

MIRRORS = {"accx_gen_params": accx.GenParams, "accx_count_opts": accx.CountOpts,
           "accx_scan_summary": accx.ScanSummary, "accx_request": accx.Request, "accx_result": accx.Result,
           "accx_server_config": accx.ServerConfig, "accx_server_stats": accx.ServerStats,
           "accx_sched_config": accx.SchedConfig, "accx_sched_info": accx.SchedInfo,
           "accx_sched_plan": accx.SchedPlan}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("layout")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "accx.h"', "int main(void) {"]
    for cname, py in MIRRORS.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["  return 0;", "}"]
    src = d / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    return {tuple(ln.split()[:2]): int(ln.split()[2]) for ln in out if ln.strip()}


@pytest.mark.parametrize("cname", sorted(MIRRORS))
def test_struct_layout_matches_the_header(c_layout, cname):
    py = MIRRORS[cname]
    assert c_layout[(cname, "size")] == ctypes.sizeof(py), cname
    for f, _ in py._fields_:
        assert c_layout[(cname, f)] == getattr(py, f).offset, (cname, f)

