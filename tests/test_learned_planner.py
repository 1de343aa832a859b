"""Learned plan scorer: its features and candidates on the CPU; on the GPU the
FP32 training gradients against the CPU oracle, BF16 inference against an
exact BF16 emulation, and the trained scorer's regret against the cost model
on held-out patterns of the recorded runtime fixture."""
import json
from pathlib import Path

import numpy as np
import pytest

from conftest import GOLDEN, PKG

FIXTURE = GOLDEN / "plan_runtimes.npz"


def test_candidates_sorted_and_first_is_the_plan(sge, graphs):
    st = graphs("chunglu_n380").stats()
    p = sge.PatternGraph.from_edges(5, [(0, 1), (0, 2), (0, 4), (1, 3), (1, 4), (2, 3)])
    c = sge.candidates(p, st, cap=32)
    assert len(c) > 4
    costs = [b.est_cost for b in c]
    assert costs == sorted(costs)
    assert c[0].to_bytes() == sge.plan(p, st).to_bytes()
    assert len({b.to_bytes() for b in c}) == len(c)


def test_features_fixed_length_and_deterministic(sge, graphs):
    st = graphs("chunglu_n380").stats()
    p = sge.PatternGraph.random(7, 17, 1)
    c = sge.candidates(p, st, cap=8)
    f = np.stack([sge.features(b, st) for b in c])
    assert f.shape == (len(c), sge.SGE_FEATURES)
    assert np.isfinite(f).all()
    assert np.array_equal(f, np.stack([sge.features(b, st) for b in c]))
    assert (f[:, 63] == 1).all()


@pytest.mark.gpu
def test_training_gradients_match_cpu_oracle(sge):
    import mlp_oracle as mo
    rng = np.random.default_rng(0)
    mlp = sge.MLP(64, 128, seed=3)
    x = rng.normal(size=(37, 64)).astype(np.float32)
    t = rng.normal(size=37).astype(np.float32)
    loss, g = mlp.loss_grad(x, t)
    want_loss, want_g = mo.loss_grad(mlp.get_params(), x, t, 64, 128)
    assert abs(loss - want_loss) <= 1e-5 * max(1.0, abs(want_loss))
    scale = np.abs(want_g).max()
    assert np.abs(g - want_g).max() <= 1e-4 * scale   # FP32 kernels vs float64
    y = mlp.forward(x)
    assert np.allclose(y, mo.forward(mlp.get_params(), x, 64, 128), rtol=1e-4, atol=1e-4)


@pytest.mark.gpu
def test_bf16_tensor_core_inference(sge):
    import mlp_oracle as mo
    rng = np.random.default_rng(1)
    mlp = sge.MLP(64, 128, seed=5)
    for B in (1, 15, 33, 200):
        x = rng.normal(size=(B, 64)).astype(np.float32)
        y = mlp.forward(x, bf16=True)
        emu = mo.forward(mlp.get_params(), x, 64, 128, bf16=True)   # BF16 operands, exact accumulation
        assert np.allclose(y, emu, rtol=2e-3, atol=2e-3), np.abs(y - emu).max()
        assert np.allclose(y, mlp.forward(x), rtol=5e-2, atol=5e-2)


@pytest.mark.gpu
def test_training_fits_a_regression(sge):
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, size=(2048, 64)).astype(np.float32)
    t = (np.sin(3 * x[:, 0]) + x[:, 1] * x[:, 2]).astype(np.float32)
    mlp = sge.MLP(64, 128, seed=7)
    first = mlp.loss_grad(x, t)[0]
    final = mlp.train(x, t, epochs=60, batch=128, lr=2e-3)
    assert final < 0.1 * first


@pytest.mark.gpu
def test_learned_scorer_beats_cost_model_on_held_out_patterns(sge):
    import sge_learn
    assert FIXTURE.exists(), "recorded runtime fixture missing"
    meta = json.loads(FIXTURE.with_suffix(".json").read_text())
    rec = sge_learn.Records.load(FIXTURE)
    train_ids = {m["id"] for m in meta["patterns"] if m["train"]}
    tr, te = sge_learn.Records(), sge_learn.Records()
    for i in range(len(rec.pattern)):
        dst = tr if rec.pattern[i] in train_ids else te
        dst.pattern.append(rec.pattern[i]); dst.cand.append(rec.cand[i]); dst.x.append(rec.x[i])
        dst.ms.append(rec.ms[i]); dst.count.append(rec.count[i])
    mlp = sge_learn.train(tr, epochs=400, seed=0)
    r = sge_learn.regret(te, mlp)
    assert r["patterns"] >= 8
    assert r["learned"] <= r["cost_model"], r
    shipped = sge_learn.load_mlp(PKG / "scorer" / "mlp_weights.npz")
    rs = sge_learn.regret(te, shipped)
    assert rs["learned"] <= rs["cost_model"], rs


@pytest.mark.gpu
def test_shipped_scorer_on_the_benchmark_setting(sge):
    """The shipped weights were trained on both recordings; on the held-out
    patterns of the R-MAT 2^22 recording (the benchmark's graph and root
    sample, tests/golden/make_plan_runtimes.py --rmat22) they pick plans no
    slower than the cost model's choice."""
    import sge_learn
    fx = GOLDEN / "plan_runtimes_rmat22.npz"
    meta = json.loads(fx.with_suffix(".json").read_text())
    rec = sge_learn.Records.load(fx)
    held = {m["id"] for m in meta["patterns"] if not m["train"]}
    te = sge_learn.Records()
    for i in range(len(rec.pattern)):
        if rec.pattern[i] in held:
            te.pattern.append(rec.pattern[i]); te.cand.append(rec.cand[i]); te.x.append(rec.x[i])
            te.ms.append(rec.ms[i]); te.count.append(rec.count[i])
    shipped = sge_learn.load_mlp(PKG / "scorer" / "mlp_weights.npz")
    rs = sge_learn.regret(te, shipped)
    assert rs["patterns"] >= 10
    assert rs["learned"] <= rs["cost_model"], rs
