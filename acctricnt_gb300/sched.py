"""Learned kernel scheduler: training data, training, tables and regret.

The cost model (accx_model, csrc/model.cu) predicts, per degree bucket and per
kernel kind (merge, gallop, bitmap), the log2 time per owned edge.  Training
data are timings the counting kernels themselves produce: for every populated
bucket and every kind, one count runs with only that bucket enabled (all other
buckets set to ACCX_KIND_SKIP) and the library's CUDA events time the counting
phases.  The same exhaustive per-bucket timing, run on a graph the model has
not seen, is the judge of the model's regret: the time its per-bucket choice
costs above the best choice per bucket.

The reference has no counterpart: it fixes the choice by a degree ratio of 50
(scan_xp_multi_gpu_multi_pass_common.cu:57-59, :105-117), the heuristic policy
here.
"""
import json
import os
import time

import numpy as np

from . import BUILD_DIR
from . import accx

NB = accx.NB
KINDS = accx.KIND_NAMES
MODEL_PATH = os.path.join(BUILD_DIR, "sched_model.json")
MODEL_PATH_ORIENTED = os.path.join(BUILD_DIR, "sched_model_oriented.json")


def _count_phase_ms(G, table, reps, stream=None, orient=False):
    best = None
    for _ in range(reps):
        G.count(policy="table", table=table, out=None, timing=True, stream=stream, orient=orient)
        ph = G.timings()
        t = ph["merge"] + ph["gallop"] + ph["bitmap"]
        best = t if best is None else min(best, t)
    return best


def bucket_timings(G, reps=2, min_edges=1, stream=None, orient=False, context=None):
    """Per-bucket timing.  Returns (edges[NB*NB], ms[NB*NB, 3]) with NaN for
    buckets not timed (fewer than min_edges owned edges).  orient=True times the
    oriented kernels on the oriented (prefix-length) buckets.

    context=None: every other bucket skipped (the bucket alone; low noise, but it
    overstates the bitmap kind, whose kernel stages an owner once for all of the
    owner's buckets -- calibrate() corrects that with a kind bias fitted on whole
    counts).  context="bitmap": the marginal cost of bucket b under kind k while
    every other populated bucket runs the bitmap kind, time(b -> k) - time(b
    skipped); on large graphs most buckets' marginal costs are below the noise of
    one whole count."""
    edges, _, _ = G.bucket_stats(orient)
    skip = np.full(NB * NB, accx.KIND_SKIP, np.uint8)
    base_table = skip.copy()
    if context == "bitmap":
        base_table[edges > 0] = accx.KIND_BITMAP
    G.count(policy="table", table=base_table, out=None, stream=stream, orient=orient)  # warm
    base_all = None
    if context is None:
        base_all = _count_phase_ms(G, skip, max(reps, 3), stream, orient)
    T = np.full((NB * NB, 3), np.nan)
    for b in np.nonzero(edges >= max(min_edges, 1))[0]:
        t = base_table.copy()
        t[b] = accx.KIND_SKIP
        base = base_all if base_all is not None else _count_phase_ms(G, t, reps, stream, orient)
        for k in range(3):
            t[b] = k
            T[b, k] = max(_count_phase_ms(G, t, reps, stream, orient) - base, 1e-4)
    return edges, T


def samples(G, edges, T, min_edges=32, orient=False):
    """Training rows: (features, kind, log2 seconds per edge)."""
    X = G.bucket_features(orient)
    xs, ks, ys = [], [], []
    for b in np.nonzero(edges >= min_edges)[0]:
        for k in range(3):
            if np.isfinite(T[b, k]):
                xs.append(X[b])
                ks.append(k)
                ys.append(np.log2(T[b, k] * 1e-3 / float(edges[b])))
    return np.array(xs, np.float32).reshape(-1, accx.MODEL_IN), np.array(ks, np.int32), np.array(ys, np.float32)


def exhaustive_table(edges, T):
    """Best kind per bucket by measurement (merge where nothing was measured)."""
    t = np.zeros(NB * NB, np.uint8)
    ok = np.isfinite(T).all(1)
    t[ok] = np.argmin(T[ok], 1)
    return t.reshape(NB, NB)


def heuristic_table(edges, sum_owner, sum_other):
    """The reference's fixed rule at bucket level: galloping when the mean
    owner degree exceeds 50 x the mean other degree, else merge."""
    t = np.zeros(NB * NB, np.uint8)
    nz = edges > 0
    mo = np.where(nz, sum_owner / np.maximum(edges, 1), 0)
    mp = np.where(nz, sum_other / np.maximum(edges, 1), 1)
    t[nz & (50 * mp < mo)] = accx.KIND_GALLOP
    return t.reshape(NB, NB)


def table_time(table, T):
    """Sum of measured per-bucket times (ms) of a table's choices."""
    tab = np.asarray(table).reshape(-1)
    ok = np.isfinite(T).all(1)
    return float(T[np.nonzero(ok)[0], tab[ok]].sum())


def regret(table, edges, T):
    best = table_time(exhaustive_table(edges, T), T)
    got = table_time(table, T)
    return {"chosen_ms": got, "best_ms": best, "regret_ms": got - best, "regret_frac": (got - best) / best if best else 0}


def training_graphs():
    return [accx.rmat_params(16, 16, seed=11), accx.rmat_params(17, 16, seed=12), accx.rmat_params(18, 16, seed=13),
            accx.rmat_params(19, 8, seed=14), accx.er_params(1 << 17, 24, seed=15),
            accx.chung_lu_params(1 << 18, 24, 2.1, 20000, seed=16), accx.chung_lu_params(1 << 17, 12, 2.5, 5000, seed=17)]


def collect(graph_params, reps=2, relabel=True, log=None, orient=False):
    xs, ks, ys = [], [], []
    for p in graph_params:
        t0 = time.perf_counter()
        G = accx.Graph.generate(p)
        if relabel:
            G.relabel()
        edges, T = bucket_timings(G, reps=reps, orient=orient)
        x, k, y = samples(G, edges, T, orient=orient)
        xs.append(x)
        ks.append(k)
        ys.append(y)
        if log:
            log("collected %d rows from n=%d m=%d in %.1f s" % (len(k), G.n, G.m, time.perf_counter() - t0))
        G.free()
    return np.concatenate(xs), np.concatenate(ks), np.concatenate(ys)


def calibration_graphs():
    return training_graphs() + [accx.rmat_params(20, 16, seed=18), accx.rmat_params(22, 16, seed=19)]


BITMAP_OFFSETS = (0.0, -0.5, -1.0, -1.5, -2.0, -3.0, -5.0, -64.0)


def calibrate(model, graph_params, orient=False, reps=3, offsets=BITMAP_OFFSETS, log=None):
    """Fits the bitmap kind's log2 offset on whole counts: for every candidate
    offset the model's table is run as a whole count on every calibration graph
    (relabeled), and the offset with the smallest size-weighted mean of times
    relative to each graph's best candidate is kept (ties: the smaller offset);
    a graph's weight is its share of the calibration set's CSR entries, so the
    large graphs decide.  -64 amounts to the bitmap kind for every bucket."""
    rel = np.zeros((len(graph_params), len(offsets)))
    wts = np.zeros(len(graph_params))
    for gi, p in enumerate(graph_params):
        G = accx.Graph.generate(p)
        G.relabel()
        wts[gi] = G.m
        for ci, off in enumerate(offsets):
            model.set_kind_bias([0.0, 0.0, off])
            rel[gi, ci] = _count_phase_ms(G, model.table_for(G, orient).reshape(-1), reps, None, orient)
        G.free()
    wts = wts / max(wts.sum(), 1.0)
    score = ((rel / rel.min(1, keepdims=True)) * wts[:, None]).sum(0) * len(graph_params)
    best = int(np.argmin(score))
    model.set_kind_bias([0.0, 0.0, offsets[best]])
    if log:
        log("calibrated bitmap offset %.2f (scores %s)" % (offsets[best], np.round(score, 3).tolist()))
    return {"kind_bias": [0.0, 0.0, float(offsets[best])], "offsets": list(offsets),
            "relative_time": [round(float(v) / len(graph_params), 4) for v in score]}


def tune_offset(G, model, orient=False, reps=2, offsets=BITMAP_OFFSETS, stream=None):
    """Refines the bitmap offset on the graph about to be counted: each candidate
    offset's model table runs once as a whole count (best of `reps`), and the
    fastest is kept in the model (ties: the calibrated offset).  The model still
    orders the kinds of every bucket; only the one trade-off scalar, which
    depends on the graph's scale, is measured in place -- as the launch-shape
    autotuner does for the bitmap kernel's shape."""
    t0 = time.perf_counter()
    base = float(model.kind_bias()[2])
    ms = []
    for off in offsets:
        model.set_kind_bias([0.0, 0.0, off])
        ms.append(_count_phase_ms(G, model.table_for(G, orient).reshape(-1), reps, stream, orient))
    best = int(np.argmin(ms))
    if base in offsets and ms[offsets.index(base)] <= ms[best]:
        best = offsets.index(base)
    model.set_kind_bias([0.0, 0.0, offsets[best]])
    return {"kind_bias": [0.0, 0.0, float(offsets[best])], "calibrated_offset": base,
            "candidate_ms": [round(float(v), 3) for v in ms], "seconds": round(time.perf_counter() - t0, 2)}


def train_default(seed=1, epochs=4000, lr=3e-3, log=None, orient=False, calibrate_bias=True):
    t0 = time.perf_counter()
    x, k, y = collect(training_graphs(), log=log, orient=orient)
    tc = time.perf_counter() - t0
    model = accx.Model(seed)
    loss0, _ = model.loss_grad(x, k, y)
    t1 = time.perf_counter()
    loss = model.train(x, k, y, epochs=epochs, lr=lr)
    info = {"rows": int(len(k)), "collect_s": round(tc, 2), "train_s": round(time.perf_counter() - t1, 2),
            "epochs": epochs, "loss_initial": loss0, "loss_final": loss}
    if calibrate_bias:
        t2 = time.perf_counter()
        info["calibration"] = calibrate(model, calibration_graphs(), orient=orient, log=log)
        info["calibration"]["seconds"] = round(time.perf_counter() - t2, 2)
    return model, info


def save(model, info, path=MODEL_PATH):
    with open(path, "w") as f:
        json.dump({"params": model.params().tolist(), "kind_bias": model.kind_bias().tolist(), "info": info}, f)


def load(path=MODEL_PATH):
    with open(path) as f:
        d = json.load(f)
    m = accx.Model(1)
    m.set_params(np.array(d["params"], np.float32))
    m.set_kind_bias(np.array(d.get("kind_bias", [0, 0, 0]), np.float32))
    return m, d["info"]


def default_model(retrain=False, log=None, orient=False):
    """The cost model of the direct (orient=False) or oriented kernels: loaded
    from the build folder, else trained on the GPU and saved there."""
    path = MODEL_PATH_ORIENTED if orient else MODEL_PATH
    if not retrain and os.path.exists(path):
        try:
            return load(path)
        except Exception:
            pass
    model, info = train_default(log=log, orient=orient)
    save(model, info, path)
    return model, info


def schedule_for(G, model=None, info=None, orient=False):
    """(table[NB][NB], info) chosen by the cost model for graph G."""
    if model is None:
        model, info = default_model(orient=orient)
    return model.table_for(G, orient), dict(info or {})


def predicted_ms(G, model, orient=False):
    """The model's predicted counting time (ms) of its own per-bucket choice:
    sum over populated buckets of edges x 2^(predicted log2 s/edge of the
    chosen kind)."""
    edges, _, _ = G.bucket_stats(orient)
    X = G.bucket_features(orient)
    nz = np.nonzero(edges > 0)[0]
    if len(nz) == 0:
        return 0.0
    y = model.predict(X[nz])
    tab = model.table_for(G, orient).reshape(-1)[nz]
    return float((edges[nz].astype(np.float64) * np.exp2(y[np.arange(len(nz)), tab].astype(np.float64))).sum() * 1e3)


def plan(G, direct_model, oriented_model):
    """Graph-level choice between direct and oriented counting by the two
    models' predicted times, each for its own per-bucket kinds."""
    pd = predicted_ms(G, direct_model, False)
    po = predicted_ms(G, oriented_model, True)
    return {"orient": po < pd, "predicted_ms": {"direct": round(pd, 3), "oriented": round(po, 3)}}
