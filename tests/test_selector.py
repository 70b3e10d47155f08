"""Technique selector: the network's GPU kernels against the float64 numpy
restatement, the analytic cost model, and AUTO's output neutrality."""
import json
import os

import numpy as np
import pytest

from conftest import ROOT


def _data(n=40, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, 12)).astype(np.float32)
    t = rng.normal(size=(n, 3)).astype(np.float32)
    m = (rng.random((n, 3)) > 0.2).astype(np.float32)
    return x, t, m


def test_numpy_reference_gradient_matches_finite_differences():
    from oracle import mlp
    from hyset_gb300.selector import init_params
    p = init_params(3).astype(np.float64)
    x, t, m = _data(10, 1)
    _, g = mlp.loss_grad(p, x, t, m)
    rng = np.random.default_rng(2)
    for i in rng.choice(p.size, 40, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-6
        num = (mlp.loss_grad(p + e, x, t, m)[0] - mlp.loss_grad(p - e, x, t, m)[0]) / 2e-6
        assert abs(num - g[i]) <= 1e-5 + 1e-4 * abs(g[i])


def test_cost_model_fit_recovers_a_linear_cost():
    from hyset_gb300.selector import cost_predict, fit_cost_model
    rng = np.random.default_rng(0)
    true = np.array([5.0, 0.1, 0.2, 0.01, 1e-5, 0.0, 1e-6, 2e-6, 0.0])
    rows = []
    for _ in range(60):
        base = [rng.uniform(1, 50), rng.uniform(5, 200), rng.uniform(1, 30), rng.uniform(1e4, 1e6),
                rng.uniform(1e4, 1e6), rng.uniform(1e5, 1e7), 0, 0]
        x = np.array([1.0, base[0], base[1], base[2], base[3], base[3] ** 2, base[4], base[5], 0.0])
        rows.append({"base": base, "ms": [float(true @ x)] * 3})
    coefs = fit_cost_model(rows)
    for r in rows[:10]:
        assert abs(cost_predict(coefs, r["base"])[1] - r["ms"][1]) <= 0.02 * r["ms"][1]


def test_shipped_selector_report_shows_the_network_gains():
    path = os.path.join(ROOT, "hyset_gb300", "selector_weights.json")
    if not os.path.exists(path):
        pytest.skip("no trained selector shipped yet")
    with open(path) as f:
        w = json.load(f)
    assert len(w["params"]) == 5187 and len(w["mean"]) == 12 and len(w["cost"]) == 27
    rep = w["report"]["held_out"]
    # held-out collections: the learned choice is at least as good as the
    # method without it (fixed rules) and as the analytic cost model
    assert rep["mlp"]["mean_regret"] <= rep["rules"]["mean_regret"] + 1e-9
    assert rep["mlp"]["mean_regret"] <= rep["cost_model"]["mean_regret"] + 1e-9


@pytest.mark.gpu
def test_gpu_forward_and_gradient_match_numpy(ctx):
    from oracle import mlp
    from hyset_gb300.selector import init_params
    for n in (5, 128, 300):  # one chunk, exactly one, several
        p = init_params(n)
        x, t, m = _data(n, n)
        y = ctx.mlp_forward(p, x)
        y64, _ = mlp.forward(p, x)
        np.testing.assert_allclose(y, y64, rtol=1e-4, atol=1e-4)
        g, loss = ctx.mlp_grad(p, x, t, m)
        l64, g64 = mlp.loss_grad(p, x, t, m)
        assert abs(loss - l64) <= 1e-4 * max(1.0, abs(l64))
        np.testing.assert_allclose(g, g64, rtol=2e-3, atol=2e-5)


@pytest.mark.gpu
def test_gpu_training_reduces_loss(ctx):
    from hyset_gb300.selector import init_params
    rng = np.random.default_rng(5)
    x = rng.normal(size=(150, 12)).astype(np.float32)
    t = np.stack([x[:, 0] * 2 - x[:, 1], np.sin(x[:, 2]), x[:, 3] ** 2], 1).astype(np.float32)
    m = np.ones_like(t)
    p, trace = ctx.mlp_train(init_params(1), x, t, m, steps=400, lr=3e-3)
    assert trace[-1] < 0.2 * trace[0]
    from oracle import mlp
    assert abs(mlp.loss_grad(p, x, t, m)[0] - trace[-1]) < 0.05 * max(trace[-1], 1e-3) + 1e-3


@pytest.mark.gpu
def test_auto_with_selector_is_output_neutral(ctx):
    import hyset_gb300 as hs
    import oracle
    from hyset_gb300 import synth
    from hyset_gb300.selector import init_params
    c = synth.generate(synth.C2, n_sets=20000, seed=4)
    coll = ctx.upload(c.tokens, c.sizes, c.starts)
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.7))
    mean, scale = np.zeros(12, np.float32), np.ones(12, np.float32)
    for bias in range(3):  # force each technique through the network's bias
        p = init_params(0)
        p[-3:] = [5.0, 5.0, 5.0]
        p[-3 + bias] = -5.0
        p[:-3] *= 0.0
        with hs.Context(0, selector=False) as c2:
            c2.selector_set(p, mean, scale, None)
            coll2 = c2.upload(c.tokens, c.sizes, c.starts)
            r = c2.self_join(coll2, threshold=0.7)
            assert r.selector == "mlp" and r.technique == ["bitmap", "fgss", "direct"][bias]
            assert oracle.as_set(r.pairs) == exp
    cost = np.zeros((3, 9))
    cost[:, 0] = [3.0, 1.0, 2.0]  # constant costs: fgss is cheapest
    with hs.Context(0, selector=False) as c3:
        c3.selector_set(None, None, None, cost)
        coll3 = c3.upload(c.tokens, c.sizes, c.starts)
        r = c3.self_join(coll3, threshold=0.7)
        assert r.selector == "cost_model" and r.technique == "fgss"
        assert oracle.as_set(r.pairs) == exp


def test_shipped_report_recomputes_from_samples():
    """The held-out regrets stored with the weights follow from the shipped
    timing samples and the network (recomputed here in float64)."""
    wpath = os.path.join(ROOT, "hyset_gb300", "selector_weights.json")
    spath = os.path.join(ROOT, "hyset_gb300", "selector_samples.json")
    if not (os.path.exists(wpath) and os.path.exists(spath)):
        pytest.skip("no trained selector shipped yet")
    from oracle import mlp
    from hyset_gb300.selector import rules_choice
    with open(wpath) as f:
        w = json.load(f)
    with open(spath) as f:
        rows = json.load(f)
    p = np.array(w["params"])
    mean, scale = np.array(w["mean"]), np.array(w["scale"])
    held = [r for r in rows if r["part"] == "all" and not r["train"]]
    assert len(held) == w["held_out"]
    x = (np.array([r["features"] for r in held]) - mean) / scale
    y, _ = mlp.forward(p, x)
    reg_mlp, reg_rules = [], []
    for r, yy in zip(held, y):
        ms = np.array(r["ms"])
        best = ms.min()
        reg_mlp.append(ms[int(np.argmin(yy))] / best - 1)
        reg_rules.append(ms[rules_choice(r)] / best - 1)
    rep = w["report"]["held_out"]
    assert abs(np.mean(reg_rules) - rep["rules"]["mean_regret"]) < 1e-3
    assert abs(np.mean(reg_mlp) - rep["mlp"]["mean_regret"]) < 0.02  # float32 GPU vs float64 argmin ties
    assert np.mean(reg_mlp) < np.mean(reg_rules)


@pytest.mark.gpu
def test_learned_partition_split_keeps_the_pairs():
    """A network that prefers the bitmap technique for short sets and the prefix
    index for long ones, and finds both dear on the whole range, splits an AUTO
    self-join into two probe ranges; the pairs stay the oracle's."""
    import hyset_gb300 as hs
    import oracle
    from hyset_gb300 import synth
    c = synth.generate(synth.C2, n_sets=60000, seed=130)
    sctx = hs.Context(0, selector=False)
    coll = sctx.upload(c.tokens, c.sizes, c.starts)
    n, mid = c.n, c.n // 2
    f_low, _ = sctx.features(coll, threshold=0.6, probe_range=(0, mid))
    f_high, _ = sctx.features(coll, threshold=0.6, probe_range=(mid, n))
    assert f_low[1] < f_high[1]
    T, L = (f_low[1] + f_high[1]) / 2, f_low[0]
    W1, b1 = np.zeros((12, 64)), np.zeros(64)
    W1[1, 0], b1[0] = 1.0, -T          # h0: the range's sets are long
    W1[1, 1], b1[1] = -1.0, T          # h1: the range's sets are short
    W1[0, 2], b1[2] = 1.0, -(L + 0.5)  # h2: more probes than a half
    W2, b2 = np.zeros((64, 64)), np.zeros(64)
    W2[0, 0] = W2[1, 1] = W2[2, 2] = 1.0
    W3, b3 = np.zeros((64, 3)), np.array([1.0, 1.0, 20.0])
    W3[0, 0] = 10.0                    # bitmap dear on long sets
    W3[1, 1] = 10.0                    # prefix index dear on short sets
    W3[2, 0] = W3[2, 1] = 8.0          # both dear on the whole range
    params = np.concatenate([a.ravel() for a in (W1, b1, W2, b2, W3, b3)]).astype(np.float32)
    sctx.selector_set(params, np.zeros(12, np.float32), np.ones(12, np.float32))
    exp = oracle.join(c.tokens, c.starts, c.sizes, 0.6)
    r = sctx.self_join(coll, threshold=0.6)
    assert r.split_at == mid and r.split_low == "bitmap" and r.technique == "fgss"
    assert r.count == len(exp) and oracle.as_set(r.pairs) == oracle.as_set(exp)
    rs = sctx.self_join(coll, threshold=0.6, sort_pairs=True)
    np.testing.assert_array_equal(rs.pairs, exp[np.lexsort((exp[:, 1], exp[:, 0]))])
    assert sctx.self_join(coll, threshold=0.6, count_only=True).count == len(exp)
    sctx.close()


@pytest.mark.gpu
def test_width_network_sets_the_signature_width():
    """A width network whose output biases favour one width makes AUTO join
    with that width (no width samples); the pairs stay the oracle's."""
    import hyset_gb300 as hs
    import oracle
    from hyset_gb300 import synth
    from hyset_gb300.selector import init_params
    c = synth.generate(synth.C2, n_sets=80000, seed=141)
    exp = oracle.as_set(oracle.join(c.tokens, c.starts, c.sizes, 0.7))
    mean, scale = np.zeros(12, np.float32), np.ones(12, np.float32)
    for k, bits in enumerate((128, 256, 512)):
        p = init_params(0)
        p[:-3] *= 0.0
        p[-3:] = [5.0, 5.0, 5.0]
        p[-3 + k] = -5.0
        with hs.Context(0, width=False) as wctx:
            wctx.width_selector_set(p, mean, scale)
            coll = wctx.upload(c.tokens, c.sizes, c.starts)
            r = wctx.self_join(coll, threshold=0.7)
            assert r.technique == "fgss" and r.bitmap_bits == bits, (bits, r.bitmap_bits)
            assert oracle.as_set(r.pairs) == exp


def test_shipped_width_report_recomputes_from_samples():
    """The width network's held-out regrets follow from its shipped timing
    samples (recomputed here in float64), and name every chooser."""
    wpath = os.path.join(ROOT, "hyset_gb300", "width_weights.json")
    spath = os.path.join(ROOT, "hyset_gb300", "width_samples.json")
    if not (os.path.exists(wpath) and os.path.exists(spath)):
        pytest.skip("no trained width network shipped yet")
    from oracle import mlp
    from hyset_gb300.width_selector import TIMED, WIDTHS, rule_bits
    with open(wpath) as f:
        w = json.load(f)
    with open(spath) as f:
        rows = json.load(f)
    held = rows[w["trained_on"]:]
    assert len(held) == w["held_out"]
    x = (np.array([r["features"] for r in held]) - np.array(w["mean"])) / np.array(w["scale"])
    y, _ = mlp.forward(np.array(w["params"]), x)
    reg_net, reg_rule = [], []
    for r, yy in zip(held, y):
        ms = dict(zip(TIMED, r["ms"]))
        best = min(ms.values())
        reg_net.append(ms[WIDTHS[int(np.argmin(yy))]] / best - 1)
        reg_rule.append(ms[rule_bits(r)] / best - 1)
    rep = w["report"]["held_out"]
    assert abs(np.mean(reg_rule) - rep["rule"]["mean_regret"]) < 1e-6
    assert abs(np.mean(reg_net) - rep["network"]["mean_regret"]) < 0.02  # float32 GPU vs float64 argmin ties
    assert set(rep) == {"network", "rule", "bits_256", "no_signatures", "autotuner"}
