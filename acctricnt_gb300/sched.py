"""Learned kernel scheduler from Python: the library's scheduler (accx_sched,
csrc/sched.cpp) plus numpy helpers that assess a schedule against measured
per-bucket timings.

Training data, training, whole-count calibration of the bitmap kind's offset,
the direct/oriented mode plan and the per-graph offset tuning all run inside
libaccx (C ABI), so the C++ drop-in and Python share one implementation.  What
stays here is analysis: the best kind per bucket by exhaustive timing, the
reference's ratio-50 rule at bucket level, and the regret of a table.

The reference has no counterpart: it fixes the choice by a degree ratio of 50
(scan_xp_multi_gpu_multi_pass_common.cu:57-59, :105-117), the heuristic policy
here.
"""
import os

import numpy as np

from . import BUILD_DIR
from . import accx

NB = accx.NB
KINDS = accx.KIND_NAMES
DEFAULT_PATH = os.path.join(BUILD_DIR, "accx-sched.model")


def count_phase_ms(G, table, reps, stream=None, orient=False):
    """Counting-phase time (merge + gallop + bitmap, ms) of a table count, best of reps."""
    best = None
    for _ in range(reps):
        G.count(policy="table", table=table, out=None, timing=True, stream=stream, orient=orient)
        ph = G.timings()
        t = ph["merge"] + ph["gallop"] + ph["bitmap"]
        best = t if best is None else min(best, t)
    return best


def bucket_timings(G, reps=2, min_edges=1, stream=None, orient=False):
    """Per-bucket timing (accx_bucket_timings): (edges[NB*NB], ms[NB*NB, 3]),
    NaN for buckets not timed; each bucket timed alone (the others skipped)."""
    return G.bucket_timings(orient=orient, reps=reps, min_edges=min_edges, stream=stream)


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


def default_scheduler(retrain=False, path=DEFAULT_PATH):
    """The scheduler in the build folder (the file SCAN_XP also reads), trained
    on the GPU and saved there when absent.  Returns (scheduler, trained_now)."""
    if not retrain and os.path.exists(path):
        try:
            return accx.Scheduler.load(path), False
        except accx.AccxError:
            pass
    s = accx.Scheduler.train()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    s.save(path)
    return s, True
