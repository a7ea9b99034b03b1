"""ctypes loader of the CPU oracle (oracle/accx_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker.  The product library never loads
it.  It also runs the reference's own CPU build (oracle/_ref/ref_harness) where
that was built, to pin the oracle against the reference.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")
REF_CLI = os.path.join(HERE, "_ref", "scan-xp-naive-bitvec")


def build(ref_root=None):
    """make -C oracle; ref_root = the reference tree (None: the Makefile's
    default); the reference build is skipped when the tree is absent."""
    args = ["make", "-s", "-C", HERE]
    if ref_root is not None:
        args.append("REF=" + ref_root)
    subprocess.run(args, check=True)


def _load():
    if not os.path.exists(LIB_PATH):
        build(ref_root=os.environ.get("ACCX_REFERENCE_ROOT", ""))
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    lib.oracle_check_graph.restype = C.c_int
    lib.oracle_check_graph.argtypes = [C.c_uint32, P, P]
    lib.oracle_cn_count.restype = C.c_int
    lib.oracle_cn_count.argtypes = [C.c_uint32, P, P, P, C.c_int]
    lib.oracle_similarity.restype = None
    lib.oracle_similarity.argtypes = [C.c_uint32, P, P, P, C.c_double, C.c_int, P, P, P, C.c_int]
    lib.oracle_cluster.restype = None
    lib.oracle_cluster.argtypes = [C.c_uint32, P, P, P, P, P]
    lib.oracle_noncore_pairs.restype = C.c_int64
    lib.oracle_noncore_pairs.argtypes = [C.c_uint32, P, P, P, P, P, P]
    lib.oracle_write_result.restype = C.c_int
    lib.oracle_write_result.argtypes = [C.c_char_p, C.c_double, C.c_int, C.c_uint32, P, P, P, C.c_int64]
    lib.oracle_eps_string.restype = None
    lib.oracle_eps_string.argtypes = [C.c_double, C.c_char_p, C.c_int]
    lib.oracle_cn_count_bitvec_stripe.restype = C.c_int64
    lib.oracle_cn_count_bitvec_stripe.argtypes = [C.c_uint32, P, P, P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]
    lib.oracle_vertex_ranges.restype = None
    lib.oracle_reorder_deg.restype = None
    lib.oracle_reorder_deg.argtypes = [C.c_uint32, P, P, C.c_int, P, P, P]
    lib.oracle_vertex_ranges.argtypes = [C.c_uint32, P, P, C.c_int, P]
    lib.oracle_sim_batch.restype = None
    lib.oracle_sim_batch.argtypes = [C.c_int64, P, P, P, C.c_double, P]
    return lib


lib = _load()


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _csr(off, dst):
    return np.ascontiguousarray(off, np.uint32), np.ascontiguousarray(dst, np.int32)


def check_graph(off, dst):
    off, dst = _csr(off, dst)
    return lib.oracle_check_graph(len(off) - 1, _p(off), _p(dst))


def cn_count(off, dst, nthreads=1):
    """common_node_num[e] = 2 + |N(u) ∩ N(v)| (CheckCoreBitmap)."""
    off, dst = _csr(off, dst)
    cnn = np.zeros(max(len(dst), 1), np.int32)
    rc = lib.oracle_cn_count(len(off) - 1, _p(off), _p(dst), _p(cnn), int(nthreads))
    if rc:
        raise RuntimeError("oracle_cn_count failed: %d" % rc)
    return cnn[:len(dst)]


REF_CHUNK = 6000  # CheckCoreBitmap's OpenMP chunk of CSR entries (scan_xp.cpp:229)


def cn_count_stripe(off, dst, cnn, stripe, nstripes, nthreads=0, chunk=REF_CHUNK):
    """One stripe of CheckCoreBitmap's entry chunks (chunks c with c % nstripes ==
    stripe), counted into cnn (int32[m], entries start at 2).  Stripes 0..nstripes-1
    together are one whole count.  Returns the CSR entries of the stripe."""
    off, dst = _csr(off, dst)
    assert cnn.dtype == np.int32 and cnn.flags.c_contiguous and len(cnn) >= len(dst)
    k = lib.oracle_cn_count_bitvec_stripe(len(off) - 1, _p(off), _p(dst), _p(cnn), int(chunk), int(stripe),
                                          int(nstripes), int(nthreads))
    if k < 0:
        raise RuntimeError("oracle_cn_count_bitvec_stripe failed: %d" % k)
    return int(k)


def reorder_deg(off, dst, nthreads=0):
    """The reference's degree-descending reorder (ReorderDegDescending + Reorder):
    returns (new_off, new_dst, old_vid) with old_vid[new id] = old id."""
    off, dst = _csr(off, dst)
    n = len(off) - 1
    new_off = np.zeros(n + 1, np.uint32)
    new_dst = np.zeros(max(len(dst), 1), np.int32)
    old_vid = np.zeros(max(n, 1), np.uint32)
    lib.oracle_reorder_deg(n, _p(off), _p(dst), int(nthreads), _p(new_off), _p(new_dst), _p(old_vid))
    return new_off, new_dst[:len(dst)], old_vid[:n]


def similarity(off, dst, cnn, eps, mu, nthreads=1):
    off, dst = _csr(off, dst)
    n = len(off) - 1
    cnn = np.ascontiguousarray(cnn, np.int32)
    sim = np.zeros(max(len(dst), 1), np.uint8)
    cc = np.zeros(max(n, 1), np.int32)
    lab = np.zeros(max(n, 1), np.int32)
    lib.oracle_similarity(n, _p(off), _p(dst), _p(cnn), float(eps), int(mu), _p(sim), _p(cc), _p(lab), int(nthreads))
    return sim[:len(dst)], cc[:n], lab[:n]


def cluster(off, dst, sim, label):
    off, dst = _csr(off, dst)
    n = len(off) - 1
    sim = np.ascontiguousarray(sim, np.uint8)
    lab = np.array(label, np.int32, copy=True)
    cl = np.zeros(max(n, 1), np.int32)
    lib.oracle_cluster(n, _p(off), _p(dst), _p(sim), _p(lab), _p(cl))
    return lab[:n], cl[:n]


def noncore_pairs(off, dst, sim, label, cl):
    off, dst = _csr(off, dst)
    n = len(off) - 1
    sim = np.ascontiguousarray(sim, np.uint8)
    label = np.ascontiguousarray(label, np.int32)
    cl = np.ascontiguousarray(cl, np.int32)
    k = lib.oracle_noncore_pairs(n, _p(off), _p(dst), _p(sim), _p(label), _p(cl), None)
    out = np.zeros(2 * max(k, 1), np.int32)
    k = lib.oracle_noncore_pairs(n, _p(off), _p(dst), _p(sim), _p(label), _p(cl), _p(out))
    return out[:2 * k].reshape(-1, 2)


def scan(off, dst, eps, mu, nthreads=1, out_dir=None):
    """The whole reference pipeline; returns a dict of arrays (and writes the
    result file into out_dir when given)."""
    cnn = cn_count(off, dst, nthreads)
    return scan_from_counts(off, dst, cnn, eps, mu, nthreads, out_dir)


def scan_from_counts(off, dst, cnn, eps, mu, nthreads=1, out_dir=None):
    """The SCAN phases after the count (similarity, cores, clusters, hubs,
    pairs, result file) on given common_node_num values."""
    sim, cc, lab0 = similarity(off, dst, cnn, eps, mu, nthreads)
    lab, cl = cluster(off, dst, sim, lab0)
    pairs = noncore_pairs(off, dst, sim, lab, cl)
    if out_dir is not None:
        p = np.ascontiguousarray(pairs.reshape(-1), np.int32)
        rc = lib.oracle_write_result(out_dir.encode(), float(eps), int(mu), len(off) - 1, _p(lab), _p(cl),
                                     _p(p) if len(p) else None, len(pairs))
        if rc:
            raise RuntimeError("oracle_write_result failed: %d" % rc)
    return {"cnn": cnn, "sim": sim, "core_count": cc, "label": lab, "cluster": cl, "pairs": pairs}


def sim_batch(cnn, du, dv, eps):
    """The reference's long double similarity test for arrays of (cnn, du, dv)."""
    cnn = np.ascontiguousarray(cnn, np.uint32)
    du = np.ascontiguousarray(du, np.uint32)
    dv = np.ascontiguousarray(dv, np.uint32)
    out = np.zeros(max(len(cnn), 1), np.uint8)
    lib.oracle_sim_batch(len(cnn), _p(cnn), _p(du), _p(dv), float(eps), _p(out))
    return out[:len(cnn)].astype(bool)


def vertex_ranges(off, dst, parts):
    off, dst = _csr(off, dst)
    r = np.zeros(parts + 1, np.uint32)
    lib.oracle_vertex_ranges(len(off) - 1, _p(off), _p(dst), int(parts), _p(r))
    return r


def eps_string(eps):
    buf = C.create_string_buffer(512)
    lib.oracle_eps_string(float(eps), buf, 512)
    return buf.value.decode()


def have_reference():
    return os.path.exists(REF_HARNESS)


def run_reference(graph_dir, eps, mu, prefix):
    """Runs the reference's own CPU build (single-threaded) on a graph directory;
    returns its dumped arrays and writes its result file into graph_dir."""
    env = dict(os.environ, OMP_NUM_THREADS="1")
    subprocess.run([REF_HARNESS, graph_dir, repr(float(eps)), str(int(mu)), prefix], check=True, env=env,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    out = {}
    for name, dt in (("cnn", np.int32), ("sim", np.uint8), ("label", np.int32), ("cluster", np.int32)):
        out[name] = np.fromfile(prefix + "." + name, dtype=dt)
    return out
