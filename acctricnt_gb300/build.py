"""Builds libaccx.so (sm_103a CUDA + C++ host code, C ABI) and the SCAN_XP CLI.

Every translation unit is compiled by nvcc for sm_103a only, in parallel, into
acctricnt_gb300/_build/.  Objects are rebuilt when a source or any header under
csrc/ or include/ is newer.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "libaccx.so")
CLIS = {"scan-xp-gb300": "main_scanxp.cpp", "scan-xp-gb300-varying": "main_scanxp_varying.cpp",
        "edge-list-to-bins-gb300": "main_edgelist.cpp", "accx-sched-train": "main_sched_train.cpp"}
CLI = os.path.join(BUILD, "scan-xp-gb300")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
              "-I" + INCLUDE, "-I" + CSRC]


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newest(paths):
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _compile(src, obj, dep_time):
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), dep_time):
        return obj, None
    cmd = [_nvcc()] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return obj, "compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr)
    return obj, None


def build(verbose=False):
    os.makedirs(os.path.join(BUILD, "obj"), exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    dep_time = _newest(headers)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    objs = []
    errors = []
    with cf.ThreadPoolExecutor(max_workers=max(2, min(len(srcs), os.cpu_count() or 4))) as ex:
        futs = []
        for s in srcs:
            obj = os.path.join(BUILD, "obj", os.path.basename(s) + ".o")
            futs.append(ex.submit(_compile, s, obj, dep_time))
        for f in futs:
            obj, err = f.result()
            objs.append(obj)
            if err:
                errors.append(err)
    if errors:
        raise RuntimeError("\n".join(errors))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest(objs):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lpthread"]
        subprocess.run(cmd, check=True)
    mains = set(CLIS.values())
    common = sorted(p for p in glob.glob(os.path.join(HOST, "*.cpp")) if os.path.basename(p) not in mains)
    host_hdrs = glob.glob(os.path.join(HOST, "*.h")) + [os.path.join(INCLUDE, "accx.h")]
    for exe, main in CLIS.items():
        out = os.path.join(BUILD, exe)
        srcs = common + [os.path.join(HOST, main)]
        if not os.path.exists(out) or os.path.getmtime(out) < max(_newest(srcs + host_hdrs), os.path.getmtime(LIB)):
            cmd = ["g++", "-O2", "-std=c++17", "-I" + INCLUDE, "-I" + HOST] + srcs + \
                ["-L" + BUILD, "-laccx", "-Wl,-rpath,$ORIGIN", "-o", out]
            subprocess.run(cmd, check=True)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
