"""The learned scheduler: the cost model's own CUDA forward/backward kernels
against a float64 CPU restatement, training, register-resident inference, the
model policy's counts (bit-exact), and its gain over the reference heuristic
assessed by exhaustive per-bucket timing on a graph it was not trained on."""
import numpy as np
import pytest

from conftest import has_gpu

pytestmark = pytest.mark.gpu

if has_gpu():
    from acctricnt_gb300 import accx, sched
    from oracle import mlp_oracle


def _rand_samples(k, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, 1, (k, accx.MODEL_IN)).astype(np.float32)
    kind = rng.integers(0, 3, k).astype(np.int32)
    y = (-27 + 3 * np.sin(3 * x[:, 0]) + 2 * x[:, 1] * kind - x[:, 2]).astype(np.float32)
    return x, kind, y


def test_gradient_matches_cpu_float64():
    m = accx.Model(seed=3)
    x, kind, y = _rand_samples(777, 1)
    loss, g = m.loss_grad(x, kind, y)
    p = m.params()  # the FP16 weights the kernels read, widened
    loss_ref, g_ref = mlp_oracle.loss_grad(p, x, kind, y)
    assert abs(loss - loss_ref) <= 1e-3 * max(1.0, abs(loss_ref))
    scale = np.abs(g_ref).max()
    assert np.max(np.abs(g - g_ref)) <= 2e-3 * scale


def test_register_resident_inference_matches_cpu():
    m = accx.Model(seed=4)
    x, _, _ = _rand_samples(1000, 2)
    y = m.predict(x)
    y_ref, _ = mlp_oracle.forward(m.params(), x)
    assert np.allclose(y, y_ref, rtol=1e-4, atol=1e-3)


def test_training_on_gpu_reduces_loss():
    m = accx.Model(seed=5)
    x, kind, y = _rand_samples(2000, 3)
    loss0, _ = m.loss_grad(x, kind, y)
    loss1 = m.train(x, kind, y, epochs=1500, lr=3e-3)
    assert loss1 < 0.1 * loss0 and loss1 < 0.5


def test_model_table_is_argmin_and_counts_are_exact():
    m = accx.Model(seed=6)
    G = accx.Graph.generate(accx.rmat_params(15, 16, seed=21))
    edges, _, _ = G.bucket_stats()
    t = m.table_for(G).reshape(-1)
    y_ref, _ = mlp_oracle.forward(m.params(), G.bucket_features())
    nz = edges > 0
    assert np.array_equal(t[nz], np.argmin(y_ref, 1)[nz])
    ref = G.count(policy="heuristic")
    G.set_model(m)
    assert np.array_equal(G.count(policy="model"), ref)
    G.relabel()
    assert np.array_equal(G.count(policy="model"), ref)


def _count_ms(G, reps=3, **kw):
    """Device time of a whole count (all phases, CUDA events), best of reps."""
    best = None
    for _ in range(reps):
        G.count(out=None, timing=True, **kw)
        t = sum(G.timings().values())
        best = t if best is None else min(best, t)
    return best


FIXED = {"direct_heuristic": dict(policy="heuristic"), "direct_merge": dict(policy="merge"),
         "direct_gallop": dict(policy="gallop"), "direct_bitmap": dict(policy="bitmap"),
         "oriented_merge": dict(policy="merge", orient=True), "oriented_gallop": dict(policy="gallop", orient=True),
         "oriented_bitmap": dict(policy="bitmap", orient=True)}


def test_scheduler_file_round_trip_and_plan(quick_sched_file, tmp_path):
    S = accx.Scheduler.load(quick_sched_file)
    with open(quick_sched_file) as f:
        assert f.readline().startswith("accx-sched 2")
    info = S.info()
    assert info["quick"]
    for mode in ("direct", "oriented"):
        assert info[mode]["rows"] > 0 and info[mode]["loss_final"] < info[mode]["loss_initial"]
        assert info[mode]["candidates"] == 1 and info[mode]["chosen"] == 0
    p2 = str(tmp_path / "again.model")
    S.save(p2)
    T = accx.Scheduler.load(p2)
    for o in (False, True):
        assert np.array_equal(S.model(o).params(), T.model(o).params())
        assert np.array_equal(S.model(o).kind_bias(), T.model(o).kind_bias())
    G = accx.Graph.generate(accx.rmat_params(15, 16, seed=31))
    ref = G.count(policy="heuristic")
    G.relabel()
    pl = S.plan(G)
    assert pl["policy"] == "model" and set(pl["predicted_ms"]) == {"direct", "oriented"}
    assert pl["orient"] == (pl["predicted_ms"]["oriented"] < pl["predicted_ms"]["direct"])
    for o in (False, True):
        assert np.array_equal(G.count(policy="model", orient=o), ref)
    with pytest.raises(accx.AccxError):
        accx.Scheduler.load(str(tmp_path / "missing.model"))


def test_version1_scheduler_files_still_load(quick_sched_file, tmp_path):
    """A version-1 file (no candidates record on the info lines) loads with the
    same models."""
    lines = open(quick_sched_file).read().splitlines()
    out = ["accx-sched 1"]
    for ln in lines[1:]:
        if ln.startswith("info "):
            ln = " ".join(ln.split()[:9 + accx.SCHED_NOFFSETS])
        out.append(ln)
    p1 = str(tmp_path / "v1.model")
    open(p1, "w").write("\n".join(out) + "\n")
    S, T = accx.Scheduler.load(quick_sched_file), accx.Scheduler.load(p1)
    for o in (False, True):
        assert np.array_equal(S.model(o).params(), T.model(o).params())
        assert np.array_equal(S.model(o).kind_bias(), T.model(o).kind_bias())
    assert T.info()["direct"]["candidates"] == 0


def test_full_training_keeps_the_best_scoring_candidate(default_sched):
    """The full scheduler trains three candidates per mode and keeps the one
    with the lowest whole-count calibration score, at its best offset."""
    info = default_sched.info()
    for mode in ("direct", "oriented"):
        d = info[mode]
        assert d["candidates"] == 3 and 0 <= d["chosen"] < 3
        sc = d["candidate_score"]
        assert len(sc) == 3 and sc[d["chosen"]] == min(sc) and sc[d["chosen"]] >= 1.0
        assert abs(min(d["calib_relative"]) - sc[d["chosen"]]) < 1e-6
        assert d["calib_relative"][accx.SCHED_OFFSETS.index(d["bitmap_offset"])] == min(d["calib_relative"])


def test_plan_tuning_keeps_a_candidate_and_counts_stay_exact(quick_sched_file):
    S = accx.Scheduler.load(quick_sched_file)
    G = accx.Graph.generate(accx.rmat_params(15, 16, seed=6))
    ref = G.count(policy="heuristic")
    G.relabel()
    pl = S.plan(G, tune=True)
    assert len(pl["tune"]["candidate_ms"]) == len(pl["tune"]["offsets"]) == accx.SCHED_NOFFSETS
    assert pl["bitmap_offset"] in pl["tune"]["offsets"]
    assert np.isclose(S.model(pl["orient"]).kind_bias()[2], pl["bitmap_offset"])
    # a tuned plan picks the mode by measurement
    assert pl["orient"] == (pl["mode_ms"]["oriented"] < pl["mode_ms"]["direct"])
    assert np.array_equal(G.count(policy="model", orient=pl["orient"]), ref)


def test_bucket_timings_cover_the_populated_buckets():
    G = accx.Graph.generate(accx.rmat_params(14, 16, seed=8))
    G.relabel()
    for orient in (False, True):
        e, T = G.bucket_timings(orient=orient, reps=1)
        pop = e > 0
        assert pop.any()
        assert np.isfinite(T[pop]).all() and (T[pop] > 0).all() and np.isnan(T[~pop]).all()


def test_learned_schedule_on_an_unseen_graph(default_sched):
    """R-MAT scale 19, seed 99 (not a training graph).  Per bucket (each bucket
    timed alone): each model's own choice beats the reference's ratio-50 rule and
    stays within 50% of the exhaustive per-bucket best.  Whole counts: the
    scheduler's plan is exact, faster than the rule, and within 10% of the
    fastest fixed single policy chosen in hindsight (every kind for every edge,
    in both modes) -- the scheduler has to find that policy without trying it."""
    S = default_sched
    G = accx.Graph.generate(accx.rmat_params(19, 16, seed=99))
    ref = G.count(policy="heuristic")
    G.relabel()
    for orient in (False, True):
        m = S.model(orient)
        edges, T = G.bucket_timings(orient=orient, reps=2)
        e, so, sp = G.bucket_stats(orient)
        heur = sched.heuristic_table(e, so, sp)
        bias = m.kind_bias()
        m.set_kind_bias([0.0, 0.0, 0.0])
        raw = m.table_for(G, orient)
        m.set_kind_bias(bias)
        assert sched.table_time(raw, T) < sched.table_time(heur, T), orient
        assert sched.regret(raw, edges, T)["regret_frac"] < 0.5, orient
    pl = S.plan(G, tune=True)
    assert np.array_equal(G.count(policy="model", orient=pl["orient"]), ref)
    t_model = _count_ms(G, policy="model", orient=pl["orient"])
    fixed = {k: _count_ms(G, **kw) for k, kw in FIXED.items()}
    assert t_model < fixed["direct_heuristic"]
    best = min(fixed.values())
    assert t_model <= 1.10 * best, (t_model, fixed)
