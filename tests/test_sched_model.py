"""The learned scheduler: the cost model's own CUDA forward/backward kernels
against a float64 CPU restatement, training, register-resident inference, the
model policy's counts (bit-exact), and its gain over the reference heuristic
judged by exhaustive per-bucket timing on a graph it was not trained on."""
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


def test_learned_schedule_beats_the_reference_heuristic_on_an_unseen_graph():
    model, info = sched.train_default(epochs=3000)
    assert info["loss_final"] < info["loss_initial"]
    G = accx.Graph.generate(accx.rmat_params(19, 16, seed=99))
    G.relabel()
    edges, T = sched.bucket_timings(G, reps=2)
    e, so, sp = G.bucket_stats()
    heur = sched.heuristic_table(e, so, sp)
    # the network's own choice (no kind offset) against buckets timed alone
    bias = model.kind_bias()
    model.set_kind_bias([0.0, 0.0, 0.0])
    raw = model.table_for(G)
    assert sched.table_time(raw, T) < sched.table_time(heur, T)
    assert sched.regret(raw, edges, T)["regret_frac"] < 0.5
    # with the offset fitted on whole counts: faster than the rule as a whole count
    model.set_kind_bias(bias)
    t_model = sched._count_phase_ms(G, model.table_for(G).reshape(-1), 3)
    t_heur = sched._count_phase_ms(G, heur.reshape(-1), 3)
    assert t_model < t_heur
