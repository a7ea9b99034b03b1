"""ctypes binding of libaccx.so (include/accx.h).

This is plumbing for tests, the bench and Python users: every call goes straight
to the C ABI, which runs the sm_103a kernels.  There is no Python or CPU
fallback: if the shared library is missing the import raises.
"""
import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libaccx.so")

OK = 0
ERR_INVALID_ARG, ERR_CUDA, ERR_OOM, ERR_SELF_LOOP, ERR_UNSORTED, ERR_RANGE, ERR_ASYMMETRIC, ERR_IO, \
    ERR_TOO_LARGE, ERR_NOT_READY, ERR_TIMEOUT, ERR_ADMISSION, ERR_NO_DEVICE = range(-1, -14, -1)

GRAPH_VALIDATE = 1
GRAPH_VALIDATE_EXACT = 2
GEN_RMAT, GEN_ER, GEN_CHUNG_LU = 0, 1, 2
KIND_MERGE, KIND_GALLOP, KIND_BITMAP = 0, 1, 2
KIND_NAMES = ("merge", "gallop", "bitmap")
POLICY_HEURISTIC, POLICY_TABLE, POLICY_MERGE, POLICY_GALLOP, POLICY_BITMAP, POLICY_MODEL = range(6)
POLICIES = {"heuristic": POLICY_HEURISTIC, "table": POLICY_TABLE, "merge": POLICY_MERGE,
            "gallop": POLICY_GALLOP, "bitmap": POLICY_BITMAP, "model": POLICY_MODEL}
NB = 24
KIND_SKIP = 3
MODEL_IN, MODEL_H, MODEL_OUT = 8, 32, 3
MODEL_NPARAMS = MODEL_IN * MODEL_H + MODEL_H + MODEL_H * MODEL_H + MODEL_H + MODEL_H * MODEL_OUT + MODEL_OUT
PHASES = ("plan", "merge", "gallop", "bitmap", "mirror")
UNCLASSIFIED, CORE, HUB = 0, 1, 2


def _validate_flags(validate):
    if validate == "exact":
        return GRAPH_VALIDATE | GRAPH_VALIDATE_EXACT
    return GRAPH_VALIDATE if validate else 0


class AccxError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        super().__init__("%s: %s (%d)" % (what, strerror(status), status))


class GenParams(C.Structure):
    _fields_ = [("kind", C.c_int), ("p0", C.c_uint64), ("p1", C.c_uint64), ("q0", C.c_double),
                ("q1", C.c_double), ("q2", C.c_double), ("seed", C.c_uint64)]


class CountOpts(C.Structure):
    _fields_ = [("policy", C.c_int), ("table", C.POINTER(C.c_uint8)), ("bias", C.c_int32),
                ("block_warps", C.c_int), ("bitmap_window_kb", C.c_int), ("timing", C.c_int), ("sparse_table_kb", C.c_int),
                ("sm_limit", C.c_int), ("orient", C.c_int)]


class ScanSummary(C.Structure):
    _fields_ = [("cores", C.c_uint32), ("clusters", C.c_uint32), ("hubs", C.c_uint32), ("outliers", C.c_uint32),
                ("similar_entries", C.c_uint64), ("noncore_pairs", C.c_uint64), ("digest", C.c_uint64)]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


REQ_QUERY, REQ_COUNT = 0, 1


class Request(C.Structure):
    _fields_ = [("type", C.c_int), ("eps", C.c_double), ("mu", C.c_int), ("graph", GenParams)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("type", C.c_int), ("queue_ms", C.c_double), ("run_ms", C.c_double),
                ("latency_ms", C.c_double), ("summary", ScanSummary), ("n", C.c_uint64), ("m", C.c_uint64),
                ("count_sum", C.c_uint64), ("count_digest", C.c_uint64)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "summary"}
        d["summary"] = self.summary.as_dict()
        return d


class ServerConfig(C.Structure):
    _fields_ = [("workers", C.c_int), ("hbm_budget", C.c_uint64), ("count_policy", C.c_int),
                ("count_sm_percent", C.c_int), ("count_orient", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("query_p50_ms", C.c_double), ("query_p99_ms", C.c_double), ("count_p50_ms", C.c_double),
                ("count_p99_ms", C.c_double), ("elapsed_s", C.c_double), ("throughput_rps", C.c_double),
                ("max_concurrent", C.c_int), ("peak_bytes", C.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


SCHED_NOFFSETS = 10
# the bitmap-kind log2 offsets the scheduler tries (kOffsets in csrc/sched.cpp)
SCHED_OFFSETS = (0.0, -0.5, -1.0, -1.5, -2.0, -3.0, -5.0, -64.0, 1.0, 64.0)
SCHED_MAX_CANDIDATES = 8


class SchedConfig(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("epochs", C.c_int), ("lr", C.c_float), ("reps", C.c_int), ("quick", C.c_int),
                ("candidates", C.c_int)]


class SchedInfo(C.Structure):
    _fields_ = [("rows", C.c_uint32 * 2), ("loss_initial", C.c_float * 2), ("loss_final", C.c_float * 2),
                ("bitmap_offset", C.c_float * 2), ("calib_relative", (C.c_float * SCHED_NOFFSETS) * 2),
                ("collect_s", C.c_double * 2), ("train_s", C.c_double * 2), ("calibrate_s", C.c_double * 2),
                ("quick", C.c_int), ("candidates", C.c_int * 2), ("chosen", C.c_int * 2),
                ("candidate_score", (C.c_float * SCHED_MAX_CANDIDATES) * 2)]


class SchedPlan(C.Structure):
    _fields_ = [("orient", C.c_int), ("predicted_ms", C.c_double * 2), ("calibrated_offset", C.c_float),
                ("bitmap_offset", C.c_float), ("tuned", C.c_int), ("offsets", C.c_float * SCHED_NOFFSETS),
                ("tune_ms", C.c_float * SCHED_NOFFSETS), ("tune_s", C.c_double), ("mode_ms", C.c_double * 2)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libaccx.so not built (run __graft_entry__.build()): %s" % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    sigs = {
        "accx_strerror": (C.c_char_p, [C.c_int]),
        "accx_version": (C.c_char_p, []),
        "accx_graph_create": (C.c_int, [P, P, C.c_uint32, C.c_uint64, C.c_uint, P, C.POINTER(P)]),
        "accx_graph_load_dir": (C.c_int, [C.c_char_p, C.c_uint, P, C.POINTER(P)]),
        "accx_graph_free": (C.c_int, [P]),
        "accx_graph_size": (C.c_int, [P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)]),
        "accx_graph_download": (C.c_int, [P, P, P, P]),
        "accx_graph_device_ptrs": (C.c_int, [P, C.POINTER(P), C.POINTER(P), C.POINTER(P)]),
        "accx_graph_generate": (C.c_int, [C.POINTER(GenParams), P, C.POINTER(P)]),
        "accx_graph_relabel": (C.c_int, [P, P]),
        "accx_graph_is_relabeled": (C.c_int, [P]),
        "accx_graph_relabeled_csr": (C.c_int, [P, P, P, P, P, P]),
        "accx_generate_host": (C.c_int, [C.POINTER(GenParams), C.POINTER(C.c_uint32), C.POINTER(C.c_uint64), P, P]),
        "accx_write_graph_dir": (C.c_int, [C.c_char_p, P, P, C.c_uint32, C.c_uint64]),
        "accx_cn_count": (C.c_int, [P, C.POINTER(CountOpts), P, P]),
        "accx_cn_last_stats": (C.c_int, [P, P, P]),
        "accx_cn_read": (C.c_int, [P, P, P]),
        "accx_cn_count_noalloc": (C.c_int, [P, P, C.c_uint32, C.c_uint64, C.c_int32, P, P]),
        "accx_cn_count_noalloc_max_entries": (C.c_uint64, []),
        "accx_cn_last_owner_work": (C.c_int, [P, P]),
        "accx_cn_last_timings": (C.c_int, [P, P]),
        "accx_scan_query": (C.c_int, [P, C.c_double, C.c_int, P, P, P, C.POINTER(ScanSummary), P]),
        "accx_scan_pairs": (C.c_int, [P, P, C.c_uint64, C.POINTER(C.c_uint64), P]),
        "accx_eps_string": (C.c_int, [C.c_double, C.c_char_p, C.c_size_t]),
        "accx_write_result": (C.c_int, [P, C.c_char_p, C.c_double, C.c_int, P]),
        "accx_similar_exact": (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_double]),
        "accx_model_create": (C.c_int, [C.c_uint64, C.POINTER(P)]),
        "accx_model_free": (C.c_int, [P]),
        "accx_model_get_params": (C.c_int, [P, P]),
        "accx_model_set_params": (C.c_int, [P, P]),
        "accx_bucket_stats": (C.c_int, [P, P, P, P]),
        "accx_bucket_features": (C.c_int, [P, P]),
        "accx_model_loss_grad": (C.c_int, [P, P, P, P, C.c_uint32, P, P]),
        "accx_model_train": (C.c_int, [P, P, P, P, C.c_uint32, C.c_int, C.c_float, P]),
        "accx_model_predict": (C.c_int, [P, P, C.c_uint32, P]),
        "accx_model_table_for": (C.c_int, [P, P, P]),
        "accx_graph_set_model": (C.c_int, [P, P]),
        "accx_cn_last_matches": (C.c_int, [P, P, P]),
        "accx_model_set_kind_bias": (C.c_int, [P, P]),
        "accx_model_get_kind_bias": (C.c_int, [P, P]),
        "accx_bucket_stats_oriented": (C.c_int, [P, P, P, P]),
        "accx_bucket_features_oriented": (C.c_int, [P, P]),
        "accx_model_table_for_oriented": (C.c_int, [P, P, P]),
        "accx_graph_set_model_oriented": (C.c_int, [P, P]),
        "accx_batch_create": (C.c_int, [P, C.c_int, P, C.POINTER(P)]),
        "accx_cn_digest": (C.c_int, [P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), P]),
        "accx_graph_from_edges": (C.c_int, [P, P, C.c_uint64, C.c_uint32, P, C.POINTER(P)]),
        "accx_triangles": (C.c_int, [P, C.POINTER(C.c_uint64), P]),
        "accx_cn_save": (C.c_int, [P, C.c_char_p]),
        "accx_cn_load": (C.c_int, [P, C.c_char_p]),
        "accx_vertex_ranges": (C.c_int, [P, C.c_int, P, P]),
        "accx_query_ctx_create": (C.c_int, [P, C.POINTER(P)]),
        "accx_query_ctx_free": (C.c_int, [P]),
        "accx_server_create": (C.c_int, [P, C.POINTER(ServerConfig), C.POINTER(P)]),
        "accx_server_submit": (C.c_int, [P, C.POINTER(Request), C.POINTER(C.c_uint64)]),
        "accx_server_poll": (C.c_int, [P, C.c_uint64, C.POINTER(Result)]),
        "accx_server_wait": (C.c_int, [P, C.c_uint64, C.c_double, C.POINTER(Result)]),
        "accx_server_drain": (C.c_int, [P]),
        "accx_server_stats_get": (C.c_int, [P, C.POINTER(ServerStats)]),
        "accx_server_request_bytes": (C.c_uint64, [P, C.POINTER(Request)]),
        "accx_server_destroy": (C.c_int, [P]),
        "accx_batch_free": (C.c_int, [P]),
        "accx_batch_union": (P, [P]),
        "accx_batch_graph_range": (C.c_int, [P, C.c_int, P, P, P, P]),
        "accx_batch_capture": (C.c_int, [P, C.POINTER(CountOpts), P]),
        "accx_batch_launch": (C.c_int, [P, P]),
        "accx_autotune": (C.c_int, [P, C.POINTER(CountOpts), C.c_int, C.POINTER(CountOpts), P, P, P, P]),
        "accx_similar_exact_batch": (C.c_int, [C.c_uint64, P, P, P, C.c_double, P]),
        "accx_bucket_timings": (C.c_int, [P, C.c_int, C.c_int, C.c_uint64, P, P, P]),
        "accx_sched_train": (C.c_int, [C.POINTER(SchedConfig), C.POINTER(P)]),
        "accx_sched_free": (C.c_int, [P]),
        "accx_sched_save": (C.c_int, [P, C.c_char_p]),
        "accx_sched_load": (C.c_int, [C.c_char_p, C.POINTER(P)]),
        "accx_sched_get_info": (C.c_int, [P, C.POINTER(SchedInfo)]),
        "accx_sched_model": (C.c_int, [P, C.c_int, C.POINTER(P)]),
        "accx_sched_plan_for": (C.c_int, [P, P, C.c_int, C.POINTER(CountOpts), C.POINTER(SchedPlan), P]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()


def strerror(status):
    return lib.accx_strerror(int(status)).decode()


def version():
    return lib.accx_version().decode()


def _check(status, what):
    if status != OK:
        raise AccxError(status, what)


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def gen_params(kind, p0, p1, q0=0.0, q1=0.0, q2=0.0, seed=1):
    return GenParams(kind, p0, p1, q0, q1, q2, seed)


def rmat_params(scale, edge_factor=16, a=0.57, b=0.19, c=0.19, seed=1):
    return gen_params(GEN_RMAT, scale, edge_factor, a, b, c, seed)


def er_params(n, mean_degree, seed=1):
    return gen_params(GEN_ER, n, int(n * mean_degree // 2), seed=seed)


def chung_lu_params(n, mean_degree, gamma=2.1, max_degree=1e6, seed=1):
    return gen_params(GEN_CHUNG_LU, n, int(n * mean_degree // 2), gamma, max_degree, seed=seed)


def generate_host(params):
    """Host generator (same graph as Graph.generate); returns (off uint32[n+1], dst int32[m])."""
    n = C.c_uint32()
    m = C.c_uint64()
    _check(lib.accx_generate_host(C.byref(params), C.byref(n), C.byref(m), None, None), "generate_host")
    off = np.zeros(n.value + 1, np.uint32)
    dst = np.zeros(max(m.value, 1), np.int32)
    _check(lib.accx_generate_host(C.byref(params), C.byref(n), C.byref(m), _ptr(off), _ptr(dst)), "generate_host")
    return off, dst[:m.value]


def write_graph_dir(path, off, dst):
    off = np.ascontiguousarray(off, np.uint32)
    dst = np.ascontiguousarray(dst, np.int32)
    _check(lib.accx_write_graph_dir(path.encode(), _ptr(off), _ptr(dst), len(off) - 1, len(dst)), "write_graph_dir")


def eps_string(eps):
    buf = C.create_string_buffer(512)
    _check(lib.accx_eps_string(float(eps), buf, 512), "eps_string")
    return buf.value.decode()


def similar_exact(cnn, du, dv, eps):
    return bool(lib.accx_similar_exact(int(cnn), int(du), int(dv), float(eps)))


def similar_exact_batch(cnn, du, dv, eps):
    cnn = np.ascontiguousarray(cnn, np.uint32)
    du = np.ascontiguousarray(du, np.uint32)
    dv = np.ascontiguousarray(dv, np.uint32)
    out = np.zeros(max(len(cnn), 1), np.uint8)
    _check(lib.accx_similar_exact_batch(len(cnn), _ptr(cnn), _ptr(du), _ptr(dv), float(eps), _ptr(out)),
           "similar_exact_batch")
    return out[:len(cnn)].astype(bool)


def cn_count_noalloc(off_ptr, dst_ptr, n, m, bias, cnt_ptr, stream=None):
    """accx_cn_count_noalloc on device pointers (no memory is allocated)."""
    _check(lib.accx_cn_count_noalloc(C.c_void_p(off_ptr), C.c_void_p(dst_ptr), int(n), int(m), int(bias),
                                     C.c_void_p(cnt_ptr), _stream_ptr(stream)), "cn_count_noalloc")


def cn_count_noalloc_max_entries():
    return int(lib.accx_cn_count_noalloc_max_entries())


def _stream_ptr(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(int(stream.cuda_stream))  # a torch.cuda.Stream


class Graph:
    """A device-resident CSR graph handle (accx_graph)."""

    def __init__(self, handle):
        self._h = handle
        n = C.c_uint32()
        m = C.c_uint64()
        _check(lib.accx_graph_size(self._h, C.byref(n), C.byref(m)), "graph_size")
        self.n, self.m = int(n.value), int(m.value)

    @classmethod
    def from_csr(cls, off, dst, validate=True, stream=None):
        """validate: True (symmetry by fingerprints), "exact" (by the sort) or False."""
        off = np.ascontiguousarray(off, np.uint32)
        dst = np.ascontiguousarray(dst, np.int32)
        h = C.c_void_p()
        _check(lib.accx_graph_create(_ptr(off), _ptr(dst) if len(dst) else None, len(off) - 1, len(dst),
                                     _validate_flags(validate), _stream_ptr(stream), C.byref(h)),
               "graph_create")
        return cls(h)

    @classmethod
    def from_device(cls, off_ptr, dst_ptr, n, m, validate=True, stream=None):
        h = C.c_void_p()
        _check(lib.accx_graph_create(C.c_void_p(off_ptr), C.c_void_p(dst_ptr), n, m,
                                     _validate_flags(validate), _stream_ptr(stream), C.byref(h)),
               "graph_create")
        return cls(h)

    @classmethod
    def load_dir(cls, path, validate=True, stream=None):
        h = C.c_void_p()
        _check(lib.accx_graph_load_dir(path.encode(), _validate_flags(validate), _stream_ptr(stream),
                                       C.byref(h)), "graph_load_dir")
        return cls(h)

    @classmethod
    def from_edges(cls, src, dst, n, stream=None):
        """Graph from an undirected edge list (the converter's job, on the device)."""
        src = np.ascontiguousarray(src, np.uint32)
        dst = np.ascontiguousarray(dst, np.uint32)
        h = C.c_void_p()
        _check(lib.accx_graph_from_edges(_ptr(src), _ptr(dst), len(src), int(n), _stream_ptr(stream), C.byref(h)),
               "graph_from_edges")
        return cls(h)

    @classmethod
    def generate(cls, params, stream=None):
        h = C.c_void_p()
        _check(lib.accx_graph_generate(C.byref(params), _stream_ptr(stream), C.byref(h)), "graph_generate")
        return cls(h)

    def relabel(self, stream=None):
        """Degree-descending relabeled copy for counting (results unchanged)."""
        _check(lib.accx_graph_relabel(self._h, _stream_ptr(stream)), "graph_relabel")

    @property
    def relabeled(self):
        return bool(lib.accx_graph_is_relabeled(self._h))

    def relabeled_csr(self):
        """(roff, rdst, map, oldid) of the relabeled copy: map[e] = the relabeled
        position of original entry e, oldid[new id] = original id."""
        n, m = self.n, self.m
        roff = np.zeros(n + 1, np.uint32)
        rdst = np.zeros(max(m, 1), np.int32)
        rmap = np.zeros(max(m, 1), np.uint32)
        oldid = np.zeros(max(n, 1), np.uint32)
        _check(lib.accx_graph_relabeled_csr(self._h, _ptr(roff), _ptr(rdst), _ptr(rmap), _ptr(oldid), None),
               "graph_relabeled_csr")
        return roff, rdst[:m], rmap[:m], oldid[:n]

    def free(self):
        if self._h and not getattr(self, "_owned_by_batch", False):
            lib.accx_graph_free(self._h)
        self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def download(self, stream=None):
        off = np.zeros(self.n + 1, np.uint32)
        dst = np.zeros(max(self.m, 1), np.int32)
        _check(lib.accx_graph_download(self._h, _ptr(off), _ptr(dst), _stream_ptr(stream)), "graph_download")
        return off, dst[:self.m]

    def device_ptrs(self):
        o, d, c = C.c_void_p(), C.c_void_p(), C.c_void_p()
        _check(lib.accx_graph_device_ptrs(self._h, C.byref(o), C.byref(d), C.byref(c)), "device_ptrs")
        return o.value, d.value, c.value

    @staticmethod
    def _opts(policy, table, bias, block_warps, window_kb, timing=False, sparse_kb=0, orient=False):
        pol = POLICIES[policy] if isinstance(policy, str) else int(policy)
        tab = None
        keep = None
        if table is not None:
            keep = np.ascontiguousarray(table, np.uint8).reshape(-1)
            assert keep.size == NB * NB
            tab = keep.ctypes.data_as(C.POINTER(C.c_uint8))
        return CountOpts(pol, tab, int(bias), int(block_warps), int(window_kb), 1 if timing else 0, int(sparse_kb),
                         0, 1 if orient else 0), keep

    def count(self, policy="heuristic", table=None, bias=0, out="host", block_warps=0, window_kb=0, stream=None,
              timing=False, sparse_kb=0, orient=False):
        """All-edge CN counts.  out="host" returns an int32 numpy array; out=None
        leaves them resident; out=<int device pointer> copies there.  orient=True
        counts triangles on prefix lists (same result, less work on a relabeled
        graph); buckets and kinds then refer to prefix lengths."""
        opts, keep = self._opts(policy, table, bias, block_warps, window_kb, timing, sparse_kb, orient)
        if out == "host":
            res = np.zeros(max(self.m, 1), np.int32)
            _check(lib.accx_cn_count(self._h, C.byref(opts), _ptr(res), _stream_ptr(stream)), "cn_count")
            return res[:self.m]
        target = None if out is None else C.c_void_p(out)
        _check(lib.accx_cn_count(self._h, C.byref(opts), target, _stream_ptr(stream)), "cn_count")
        del keep
        return None

    def digest(self, stream=None):
        """(sum, order-independent hash) of the resident counts."""
        a, b = C.c_uint64(), C.c_uint64()
        _check(lib.accx_cn_digest(self._h, C.byref(a), C.byref(b), _stream_ptr(stream)), "cn_digest")
        return int(a.value), int(b.value)

    def triangles(self, stream=None):
        t = C.c_uint64()
        _check(lib.accx_triangles(self._h, C.byref(t), _stream_ptr(stream)), "triangles")
        return int(t.value)

    def save_counts(self, path):
        _check(lib.accx_cn_save(self._h, path.encode()), "cn_save")

    def load_counts(self, path):
        _check(lib.accx_cn_load(self._h, path.encode()), "cn_load")

    def vertex_ranges(self, parts, stream=None):
        r = np.zeros(parts + 1, np.uint32)
        _check(lib.accx_vertex_ranges(self._h, int(parts), _ptr(r), _stream_ptr(stream)), "vertex_ranges")
        return r

    def read_counts(self, stream=None):
        """The resident counts (after a count or a captured replay), to the host."""
        res = np.zeros(max(self.m, 1), np.int32)
        _check(lib.accx_cn_read(self._h, _ptr(res), _stream_ptr(stream)), "cn_read")
        return res[:self.m]

    def last_stats(self):
        e = np.zeros(3, np.uint64)
        w = np.zeros(3, np.uint64)
        _check(lib.accx_cn_last_stats(self._h, _ptr(e), _ptr(w)), "cn_last_stats")
        return {KIND_NAMES[k]: {"edges": int(e[k]), "work": int(w[k])} for k in range(3)}

    def last_matches(self):
        """Oriented counts: (common ids found per kind, ids probed by the bitmap kind)."""
        mt = np.zeros(3, np.uint64)
        pr = C.c_uint64()
        _check(lib.accx_cn_last_matches(self._h, _ptr(mt), C.byref(pr)), "cn_last_matches")
        return {KIND_NAMES[k]: int(mt[k]) for k in range(3)}, int(pr.value)

    def owner_work(self):
        w = np.zeros(3, np.uint64)
        _check(lib.accx_cn_last_owner_work(self._h, _ptr(w)), "cn_last_owner_work")
        return {KIND_NAMES[k]: int(w[k]) for k in range(3)}

    def timings(self):
        """Milliseconds per phase (plan, merge, gallop, bitmap, mirror) of the last timed count."""
        ms = np.zeros(5, np.float32)
        _check(lib.accx_cn_last_timings(self._h, _ptr(ms)), "cn_last_timings")
        return dict(zip(PHASES, (float(x) for x in ms)))

    def autotune(self, policy="bitmap", reps=2, stream=None, orient=False):
        """Fastest bitmap-kernel launch shape for `policy`; returns (kwargs, ms, all_ms)."""
        base, keep = self._opts(policy, None, 0, 0, 0, False, 0, orient)
        best = CountOpts()
        bms = C.c_float()
        allms = np.zeros(16, np.float32)
        nc = C.c_int()
        _check(lib.accx_autotune(self._h, C.byref(base), int(reps), C.byref(best), C.byref(bms), _ptr(allms),
                                 C.byref(nc), _stream_ptr(stream)), "autotune")
        return ({"block_warps": best.block_warps, "window_kb": best.bitmap_window_kb,
                 "sparse_kb": best.sparse_table_kb}, float(bms.value), allms[:nc.value].tolist())

    def bucket_stats(self, orient=False):
        """Per-bucket owned edges and owner / other size sums; orient=True uses
        prefix lengths on the counting CSR (the oriented buckets)."""
        e = np.zeros(NB * NB, np.uint64)
        so = np.zeros(NB * NB, np.float64)
        sp = np.zeros(NB * NB, np.float64)
        fn = lib.accx_bucket_stats_oriented if orient else lib.accx_bucket_stats
        _check(fn(self._h, _ptr(e), _ptr(so), _ptr(sp)), "bucket_stats")
        return e, so, sp

    def bucket_timings(self, orient=False, reps=2, min_edges=1, stream=None):
        """Per-bucket kernel timings (accx_bucket_timings): (edges[NB*NB],
        ms[NB*NB, 3]) with NaN for buckets not timed."""
        e = np.zeros(NB * NB, np.uint64)
        t = np.zeros(NB * NB * 3, np.float32)
        _check(lib.accx_bucket_timings(self._h, 1 if orient else 0, int(reps), int(min_edges), _ptr(e), _ptr(t),
                                       _stream_ptr(stream)), "bucket_timings")
        return e, t.reshape(NB * NB, 3).astype(np.float64)

    def bucket_features(self, orient=False):
        x = np.zeros((NB * NB, MODEL_IN), np.float32)
        fn = lib.accx_bucket_features_oriented if orient else lib.accx_bucket_features
        _check(fn(self._h, _ptr(x)), "bucket_features")
        return x

    def set_model(self, model, orient=False):
        """Attach the model ACCX_POLICY_MODEL uses (for direct or oriented counts)."""
        if orient:
            self._model_or = model  # keep the model alive while attached
            _check(lib.accx_graph_set_model_oriented(self._h, model._h if model else None), "graph_set_model")
        else:
            self._model = model
            _check(lib.accx_graph_set_model(self._h, model._h if model else None), "graph_set_model")

    def scan(self, eps, mu, want_sim=True, want_label=True, want_cluster=True, stream=None):
        sim = np.zeros(max(self.m, 1), np.uint8) if want_sim else None
        lab = np.zeros(max(self.n, 1), np.int32) if want_label else None
        cl = np.zeros(max(self.n, 1), np.int32) if want_cluster else None
        s = ScanSummary()
        _check(lib.accx_scan_query(self._h, float(eps), int(mu), _ptr(sim), _ptr(lab), _ptr(cl), C.byref(s),
                                   _stream_ptr(stream)), "scan_query")
        return {"sim": None if sim is None else sim[:self.m], "label": None if lab is None else lab[:self.n],
                "cluster": None if cl is None else cl[:self.n], "summary": s.as_dict()}

    def pairs(self, stream=None):
        k = C.c_uint64()
        _check(lib.accx_scan_pairs(self._h, None, 0, C.byref(k), _stream_ptr(stream)), "scan_pairs")
        out = np.zeros(2 * max(k.value, 1), np.int32)
        _check(lib.accx_scan_pairs(self._h, _ptr(out), k.value, C.byref(k), _stream_ptr(stream)), "scan_pairs")
        return out[:2 * k.value].reshape(-1, 2)

    def write_result(self, path, eps, mu, stream=None):
        _check(lib.accx_write_result(self._h, path.encode(), float(eps), int(mu), _stream_ptr(stream)), "write_result")


class Model:
    """The MLP cost model (accx_model): FP16 weights on the device."""

    def __init__(self, seed=1):
        self._h = C.c_void_p()
        self._owner = None
        _check(lib.accx_model_create(int(seed), C.byref(self._h)), "model_create")

    @classmethod
    def _borrowed(cls, handle, owner):
        """A model owned by a scheduler (freed with it)."""
        m = cls.__new__(cls)
        m._h = handle
        m._owner = owner
        return m

    def __del__(self):
        try:
            if self._h and self._owner is None:
                lib.accx_model_free(self._h)
            self._h = None
        except Exception:
            pass

    def params(self):
        p = np.zeros(MODEL_NPARAMS, np.float32)
        _check(lib.accx_model_get_params(self._h, _ptr(p)), "model_get_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == MODEL_NPARAMS
        _check(lib.accx_model_set_params(self._h, _ptr(p)), "model_set_params")

    @staticmethod
    def _samples(x, kind, target):
        return (np.ascontiguousarray(x, np.float32).reshape(-1, MODEL_IN), np.ascontiguousarray(kind, np.int32),
                np.ascontiguousarray(target, np.float32))

    def loss_grad(self, x, kind, target):
        x, kind, target = self._samples(x, kind, target)
        g = np.zeros(MODEL_NPARAMS, np.float32)
        loss = C.c_float()
        _check(lib.accx_model_loss_grad(self._h, _ptr(x), _ptr(kind), _ptr(target), len(kind), _ptr(g),
                                        C.byref(loss)), "model_loss_grad")
        return float(loss.value), g

    def train(self, x, kind, target, epochs=2000, lr=3e-3):
        x, kind, target = self._samples(x, kind, target)
        loss = C.c_float()
        _check(lib.accx_model_train(self._h, _ptr(x), _ptr(kind), _ptr(target), len(kind), int(epochs), float(lr),
                                    C.byref(loss)), "model_train")
        return float(loss.value)

    def kind_bias(self):
        b = np.zeros(MODEL_OUT, np.float32)
        _check(lib.accx_model_get_kind_bias(self._h, _ptr(b)), "model_get_kind_bias")
        return b

    def set_kind_bias(self, bias):
        b = np.ascontiguousarray(bias, np.float32).reshape(MODEL_OUT)
        _check(lib.accx_model_set_kind_bias(self._h, _ptr(b)), "model_set_kind_bias")

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, MODEL_IN)
        y = np.zeros((len(x), MODEL_OUT), np.float32)
        _check(lib.accx_model_predict(self._h, _ptr(x), len(x), _ptr(y)), "model_predict")
        return y

    def table_for(self, graph, orient=False):
        t = np.zeros(NB * NB, np.uint8)
        fn = lib.accx_model_table_for_oriented if orient else lib.accx_model_table_for
        _check(fn(self._h, graph._h, _ptr(t)), "model_table_for")
        return t.reshape(NB, NB)


class Scheduler:
    """The learned scheduler (accx_sched): a direct and an oriented cost model,
    trained, calibrated, saved and planned by the library."""

    def __init__(self, handle):
        self._h = handle

    @classmethod
    def train(cls, seed=1, epochs=0, lr=0.0, reps=0, quick=False, candidates=0):
        h = C.c_void_p()
        cfg = SchedConfig(int(seed), int(epochs), float(lr), int(reps), 1 if quick else 0, int(candidates))
        _check(lib.accx_sched_train(C.byref(cfg), C.byref(h)), "sched_train")
        return cls(h)

    @classmethod
    def load(cls, path):
        h = C.c_void_p()
        _check(lib.accx_sched_load(path.encode(), C.byref(h)), "sched_load")
        return cls(h)

    def save(self, path):
        _check(lib.accx_sched_save(self._h, path.encode()), "sched_save")

    def free(self):
        if self._h:
            lib.accx_sched_free(self._h)
        self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def model(self, orient=False):
        h = C.c_void_p()
        _check(lib.accx_sched_model(self._h, 1 if orient else 0, C.byref(h)), "sched_model")
        return Model._borrowed(h, self)

    def info(self):
        i = SchedInfo()
        _check(lib.accx_sched_get_info(self._h, C.byref(i)), "sched_get_info")
        out = {}
        for o, mode in enumerate(("direct", "oriented")):
            out[mode] = {"rows": int(i.rows[o]), "loss_initial": round(float(i.loss_initial[o]), 4),
                         "loss_final": round(float(i.loss_final[o]), 4),
                         "bitmap_offset": float(i.bitmap_offset[o]),
                         "calib_relative": [round(float(x), 4) for x in i.calib_relative[o]],
                         "collect_s": round(i.collect_s[o], 2), "train_s": round(i.train_s[o], 2),
                         "calibrate_s": round(i.calibrate_s[o], 2), "candidates": int(i.candidates[o]),
                         "chosen": int(i.chosen[o]),
                         "candidate_score": [round(float(x), 4) for x in i.candidate_score[o][:max(int(i.candidates[o]), 0)]]}
        out["quick"] = bool(i.quick)
        return out

    def plan(self, graph, tune=False, stream=None):
        """Attaches both models to `graph` and picks the mode; returns a dict with
        "policy" ("model"), "orient" and the predictions (and tuning times)."""
        o = CountOpts()
        p = SchedPlan()
        _check(lib.accx_sched_plan_for(self._h, graph._h, 1 if tune else 0, C.byref(o), C.byref(p),
                                       _stream_ptr(stream)), "sched_plan_for")
        graph._model = self.model(False)
        graph._model_or = self.model(True)
        graph._sched = self
        d = {"policy": "model", "orient": bool(p.orient),
             "predicted_ms": {"direct": round(p.predicted_ms[0], 3), "oriented": round(p.predicted_ms[1], 3)},
             "calibrated_offset": float(p.calibrated_offset), "bitmap_offset": float(p.bitmap_offset)}
        if p.tuned:
            d["mode_ms"] = {"direct": round(p.mode_ms[0], 3), "oriented": round(p.mode_ms[1], 3)}
            d["tune"] = {"offsets": [float(x) for x in p.offsets], "candidate_ms": [round(float(x), 3) for x in p.tune_ms],
                         "seconds": round(p.tune_s, 2)}
        return d


class Batch:
    """K graphs joined into one disjoint-union CSR (accx_batch)."""

    def __init__(self, graphs, stream=None):
        self.graphs = list(graphs)
        arr = (C.c_void_p * len(self.graphs))(*[g._h for g in self.graphs])
        self._h = C.c_void_p()
        _check(lib.accx_batch_create(arr, len(self.graphs), _stream_ptr(stream), C.byref(self._h)), "batch_create")
        u = Graph.__new__(Graph)
        u._h = C.c_void_p(lib.accx_batch_union(self._h))
        n = C.c_uint32()
        m = C.c_uint64()
        _check(lib.accx_graph_size(u._h, C.byref(n), C.byref(m)), "graph_size")
        u.n, u.m = int(n.value), int(m.value)
        u._owned_by_batch = True
        self.union = u
        self.ranges = []
        for i in range(len(self.graphs)):
            vb, nn, eb, mm = C.c_uint32(), C.c_uint32(), C.c_uint64(), C.c_uint64()
            _check(lib.accx_batch_graph_range(self._h, i, C.byref(vb), C.byref(nn), C.byref(eb), C.byref(mm)),
                   "batch_graph_range")
            self.ranges.append((int(vb.value), int(nn.value), int(eb.value), int(mm.value)))

    def free(self):
        if self._h:
            self.union._h = None  # owned by the batch
            lib.accx_batch_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass

    def capture(self, policy="model", bias=0, stream=None, **kw):
        opts, keep = Graph._opts(policy, None, bias, kw.get("block_warps", 0), kw.get("window_kb", 0), False,
                                 kw.get("sparse_kb", 0), kw.get("orient", False))
        _check(lib.accx_batch_capture(self._h, C.byref(opts), _stream_ptr(stream)), "batch_capture")

    def launch(self, stream=None):
        _check(lib.accx_batch_launch(self._h, _stream_ptr(stream)), "batch_launch")

    def split(self, arr, per="entry"):
        """Slices of a union-wide array per graph (per entry or per vertex)."""
        out = []
        for vb, n, eb, m in self.ranges:
            out.append(arr[eb:eb + m] if per == "entry" else arr[vb:vb + n])
        return out


def query_request(eps, mu):
    return Request(REQ_QUERY, float(eps), int(mu), GenParams())


def count_request(params):
    return Request(REQ_COUNT, 0.0, 0, params)


class Server:
    """accx_server: continuous batching of SCAN queries on a resident counted
    graph and of new-graph count requests, admitted by an HBM budget."""

    def __init__(self, resident, workers=4, hbm_budget=0, count_policy="bitmap", count_sm_percent=0,
                 count_orient=False):
        self.resident = resident
        pol = POLICIES[count_policy] if isinstance(count_policy, str) else int(count_policy)
        cfg = ServerConfig(int(workers), int(hbm_budget), pol, int(count_sm_percent), 1 if count_orient else 0)
        self._h = C.c_void_p()
        _check(lib.accx_server_create(resident._h, C.byref(cfg), C.byref(self._h)), "server_create")

    def submit(self, req):
        i = C.c_uint64()
        _check(lib.accx_server_submit(self._h, C.byref(req), C.byref(i)), "server_submit")
        return int(i.value)

    def poll(self, rid):
        r = Result()
        st = lib.accx_server_poll(self._h, int(rid), C.byref(r))
        if st == ERR_NOT_READY:
            return None
        _check(st, "server_poll")
        return r

    def wait(self, rid, timeout_ms=-1.0):
        r = Result()
        _check(lib.accx_server_wait(self._h, int(rid), float(timeout_ms), C.byref(r)), "server_wait")
        return r

    def drain(self):
        _check(lib.accx_server_drain(self._h), "server_drain")

    def stats(self):
        st = ServerStats()
        _check(lib.accx_server_stats_get(self._h, C.byref(st)), "server_stats")
        return st.as_dict()

    def request_bytes(self, req):
        return int(lib.accx_server_request_bytes(self._h, C.byref(req)))

    def close(self):
        if self._h:
            lib.accx_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
