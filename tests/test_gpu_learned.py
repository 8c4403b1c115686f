"""The learned cost model: hand-written kernels vs the numpy oracle, training, and the
schedule it drives (which must never change a count)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle.mlp_ref as M

pytestmark = pytest.mark.gpu


def test_forward_and_gradient_match_oracle(xgm, ctx):
    rng = np.random.default_rng(0)
    m = xgm.Model(ctx, seed=3)
    p = (rng.standard_normal(xgm.MODEL_PARAMS) * 0.4).astype(np.float32)
    m.set_params(p)
    X = rng.random((3000, xgm.MODEL_FEATURES)).astype(np.float32)
    y = (rng.random(3000) * 8).astype(np.float32)
    # forward: fp16 weights, fp32 accumulation; tolerance covers fp32 vs fp64 sums
    np.testing.assert_allclose(m.predict(X), M.forward(p, X), rtol=1e-4, atol=1e-4)
    loss, g = m.loss_grad(X, y)
    rl, rg = M.loss_grad(p, X, y)
    assert abs(loss - rl) <= 1e-4 * max(1.0, abs(rl))
    # gradient: float atomics reorder sums; relative 1e-3 of the largest component
    np.testing.assert_allclose(g, rg, rtol=1e-3, atol=1e-3 * np.abs(rg).max())


def test_training_reduces_loss(xgm, ctx):
    rng = np.random.default_rng(1)
    X = rng.random((20000, xgm.MODEL_FEATURES)).astype(np.float32)
    w = rng.standard_normal(xgm.MODEL_FEATURES)
    y = (10 + 4 * np.tanh(X @ w)).astype(np.float32)
    m = xgm.Model(ctx, seed=2)
    l0, _ = m.loss_grad(X, y)
    l1 = m.train(X, y, epochs=15, batch=512, lr=3e-3)
    assert l1 < 0.1 * l0


def test_collect_and_learned_schedule_counts(xgm, ctx):
    nv, s, d = xgm.gen_rmat(14, 16, seed=41)
    g = ctx.graph_from_edges(nv, s, d)
    m = xgm.Model(ctx, seed=4)
    Xs, ys = [], []
    for var in xgm.ALL_VARIANTS:
        X, y, cnt = m.collect(g, "4-clique", var, stride=2, max_rows=50000)
        assert cnt == ctx.count(g, "4-clique")
        assert len(y) > 0 and np.all(np.isfinite(X)) and np.all(np.isfinite(y))
        assert np.all(X[:, 5 + var] == 1.0)  # one-hot after 4 shape features + depth
        Xs.append(X)
        ys.append(y)
    m.train(np.concatenate(Xs), np.concatenate(ys), epochs=10)
    for pat in ("triangle", "4-clique", "5-clique", "diamond", "tailedtriangle"):
        base = ctx.count(g, pat)
        assert ctx.count(g, pat, policy=xgm.SCHED_LEARNED, model=m) == base
        assert ctx.count(g, pat, policy=xgm.SCHED_LEARNED, model=m, order_by_cost=0) == base


def test_learned_schedule_in_batches(xgm, ctx):
    vo, eo, s, d = xgm.gen_ba_batch(32, 100, 2000, 3, 8, seed=8)
    b = ctx.batch_from_edges(vo, s, d)
    m = xgm.Model(ctx, seed=5)
    base = ctx.count_batched(b, ["triangle", "4-clique", "diamond"])
    got = ctx.count_batched(b, ["triangle", "4-clique", "diamond"], policy=xgm.SCHED_LEARNED,
                            model=m)
    assert np.array_equal(base, got)


def test_trained_model_gains_on_held_out_graph(xgm, ctx):
    """The trained cost model (costmodel.json) against the plain degree-threshold
    heuristic on a graph outside its training and validation sets (R-MAT scale 21, seed
    77; training used seeds 10-14, validation seed 98, evaluation seed 99): same count,
    and the learned schedule is not slower (best of 5 counts each; 3 % tolerance for
    timing noise; it measured ~5 % faster at scale 22 and ~8 % at scale 23)."""
    learned = xgm.trained_schedule(ctx)
    if not learned:
        pytest.skip("costmodel.json absent")
    nv, s, d = xgm.gen_rmat(21, 16, seed=77)
    g = ctx.graph_from_edges(nv, s, d)

    def best(kw):
        ctx.count(g, "4-clique", **kw)
        ms, cnt = [], None
        for _ in range(5):
            cnt, st = ctx.count(g, "4-clique", with_stats=True, **kw)
            ms.append(st["kernel_ms"] + st["prep_ms"])
        return cnt, min(ms)

    c_h, t_h = best({})
    c_l, t_l = best(learned)
    assert c_l == c_h
    assert t_l <= 1.03 * t_h, f"learned {t_l:.2f} ms vs plain heuristic {t_h:.2f} ms"
    g.close()
