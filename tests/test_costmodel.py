"""The learned matching-order cost model (a 32-64-64-1 MLP with BF16 weights, trained on the GPU).

CPU: the numpy oracle's backpropagation equals central finite differences (without BF16 rounding).
GPU: the hand-written kernels' predictions and gradients equal the oracle's (same BF16 rounding
points; FP32 vs float64 sums and the order of atomic adds are the only differences, hence the
tolerances); Adam training lowers the loss; and a model trained on records the plain miner logs on
configuration 1-3 graphs chooses, on the held-out configuration-5 graph, orders that keep the
reference's pattern set and exact supports and cut the search steps.
"""
from __future__ import annotations

import importlib.util
import sys

import numpy as np
import pytest

from conftest import ROOT, has_gpu

spec = importlib.util.spec_from_file_location("mlp_oracle", ROOT / "oracle" / "mlp_oracle.py")
mlp_oracle = importlib.util.module_from_spec(spec)
sys.modules["mlp_oracle"] = mlp_oracle
spec.loader.exec_module(mlp_oracle)


def random_problem(seed, n):
    rng = np.random.default_rng(seed)
    p = np.zeros(mlp_oracle.N_PARAMS, dtype=np.float32)
    w1, b1, w2, b2, w3, b3 = (slice(0, 2048), slice(2048, 2112), slice(2112, 6208), slice(6208, 6272),
                              slice(6272, 6336), slice(6336, 6337))
    p[w1] = rng.uniform(-0.4, 0.4, 2048)
    p[b1] = rng.uniform(-0.1, 0.1, 64)
    p[w2] = rng.uniform(-0.3, 0.3, 4096)
    p[b2] = rng.uniform(-0.1, 0.1, 64)
    p[w3] = rng.uniform(-0.3, 0.3, 64)
    p[b3] = 0.5
    x = rng.uniform(0, 1, (n, 32)).astype(np.float32)
    t = rng.uniform(0, 4, n).astype(np.float32)
    return p, x, t


def test_oracle_gradient_equals_finite_differences():
    p, x, t = random_problem(1, 23)
    p = p.astype(np.float64)
    g = mlp_oracle.gradients(p.astype(np.float32), x, t, rounding=False)
    rng = np.random.default_rng(2)
    for i in rng.choice(len(p), 60, replace=False):
        h = 1e-3
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        # loss in float64 on float32-rounded parameters: use a step large enough to survive rounding
        fd = (mlp_oracle.loss(pp.astype(np.float32), x, t, False) - mlp_oracle.loss(pm.astype(np.float32), x, t, False)) / (
            (pp[i].astype(np.float32) - pm[i].astype(np.float32)))
        assert abs(fd - g[i]) <= 2e-3 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.01171875, -3.5, 1e-30, 65504.0], dtype=np.float32)
    r = mlp_oracle.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625 and r[3] == -3.5
    assert np.all(np.abs(r - v) <= np.abs(v) * 2 ** -8)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [16, 100, 1000])
def test_gpu_forward_and_gradients_equal_oracle(tfsm, n):
    p, x, t = random_problem(n, n)
    m = tfsm.CostModel(seed=0)
    try:
        m.set_params(p)
        y = m.predict(x)
        y_ref, _ = mlp_oracle.forward(p, x)
        assert np.allclose(y, y_ref, rtol=1e-3, atol=1e-3 * np.abs(y_ref).max()), np.abs(y - y_ref).max()
        g = m.gradients(x, t)
        g_ref = mlp_oracle.gradients(p, x, t)
        scale = np.abs(g_ref).max()
        err = np.abs(g - g_ref)
        # BF16 rounding of dZ2 / dZ1 may fall on the other side of a tie between FP32 and float64
        assert err.max() <= 1e-2 * scale, (err.max(), scale)
        assert np.mean(err) <= 1e-3 * scale
    finally:
        m.close()


@pytest.mark.gpu
def test_gpu_training_lowers_loss(tfsm):
    rng = np.random.default_rng(7)
    x = rng.uniform(0, 1, (4000, 32)).astype(np.float32)
    t = (3 * x[:, 3] + 2 * x[:, 7] * x[:, 12] + np.sin(4 * x[:, 20])).astype(np.float32)
    m = tfsm.CostModel(seed=3)
    try:
        before = mlp_oracle.loss(m.params(), x, t)
        after = m.train(x, t, epochs=30, batch=128, lr=2e-3, seed=1)
        assert after < 0.1 * before, (before, after)
        assert abs(after - mlp_oracle.loss(m.params(), x, t)) <= 0.05 * after + 1e-3
    finally:
        m.close()


def _gen(built, out, gen: dict, seed: int):
    import subprocess

    args = [str(built / "bin" / "gen_lg"), "--out", str(out)]
    for k, v in dict(gen, seed=seed).items():
        args += ["--" + k.replace("_", "-"), str(v)]
    subprocess.run(args, check=True, capture_output=True)
    return out


# graph shapes of the benchmark configurations (configuration 3 is the configuration-2 graph at tau 5000)
SHAPE_C1 = dict(n=5000, mean=8, gamma=2.5, max_degree=500, labels=10, zipf=1.0, elabels=1)
SHAPE_C2 = dict(n=100000, mean=22, gamma=2.2, max_degree=1400, labels=29, zipf=1.2, elabels=1)


def _train_on_configs_1_to_3(tfsm, built, tmp_path):
    """Records of the plain miner with seeded random orders: configuration 1 (seeds 10-19, tau 200,
    4 vertices), configuration 2 (seeds 10-13, tau 9000, 5 vertices) and configuration 3's tau on
    the configuration-2 shape (seeds 14-15, tau 5000, 5 vertices)."""
    train = [(SHAPE_C1, s, 200, 4) for s in range(10, 20)] + [(SHAPE_C2, s, 9000, 5) for s in range(10, 14)] + \
            [(SHAPE_C2, s, 5000, 5) for s in (14, 15)]
    feats, costs = [], []
    for k, (shape, seed, tau, max_nodes) in enumerate(train):
        path = _gen(built, tmp_path / f"train_{shape['n']}_{seed}.lg", shape, seed)
        with tfsm.Graph.load(path, tau) as g:
            g.set_order_policy(tfsm.ORDER_RANDOM, seed=k + 1)
            g.record_orders(True)
            g.mine(max_nodes=max_nodes, flags=tfsm.FLAG_PLAIN)
            f, c = g.take_records()
            feats.append(f)
            costs.append(c)
    return np.concatenate(feats), np.concatenate(costs)


def _mine(tfsm, path, tau, max_nodes, policy, model, out):
    with tfsm.Graph.load(path, tau) as g:
        g.set_order_policy(policy, model=model if policy == tfsm.ORDER_MODEL else None)
        st = g.mine(max_nodes=max_nodes, results_path=out)
        keys = sorted(set(tfsm.read_results(out)))
        return g, st, keys


@pytest.mark.gpu
def test_learned_orders_on_held_out_config5_graph(tfsm, built, tmp_path, case_graph):
    """The model trained on configurations 1-3 (seeds 10-19) chooses the matching orders on the
    held-out seed-99 graph of configuration 5.

    * tau 20000, maxNodes 5 (configuration 5): the reference's pattern set (golden) and the golden
      exact MNI of every candidate the reference's harness evaluated;
    * tau 5000, maxNodes 5 (the same graph where searches are long): the GQL order's pattern set and
      exact supports (a sample of 60 frequent patterns), with fewer search steps: the median of
      three mining runs per order at least 1.2x lower (measured 1.4x to 5.3x; the GQL order's step
      count varies from run to run with which search finds an embedding first, the model's less).
    The measured gains are printed."""
    import json

    from conftest import golden_mni, golden_pattern_set

    x, t = _train_on_configs_1_to_3(tfsm, built, tmp_path)
    assert len(x) >= 2000, len(x)
    m = tfsm.CostModel(seed=1)
    try:
        mse0 = mlp_oracle.loss(m.params(), x, t)
        mse = m.train(x, t, epochs=60, batch=64, lr=2e-3, seed=2)
        assert mse < 0.5 * mse0, (mse0, mse)
        held = case_graph("cfg5_seed99")
        summary = {"records": int(len(x)), "train_mse": [mse0, mse]}
        # configuration 5 as written
        _, st20, keys20 = _mine(tfsm, held, 20000, 5, tfsm.ORDER_MODEL, m, tmp_path / "m20.txt")
        assert set(keys20) == golden_pattern_set("cfg5_seed99")
        want = golden_mni("cfg5_seed99")
        with tfsm.Graph.load(held, 20000) as g:
            g.set_order_policy(tfsm.ORDER_MODEL, model=m)
            got = g.evaluate([tfsm.parse_key(k) for k in want], flags=tfsm.FLAG_EXACT)
        assert {k: r.mni for k, r in zip(want, got)} == want
        _, gst20, _ = _mine(tfsm, held, 20000, 5, tfsm.ORDER_GQL, None, tmp_path / "g20.txt")
        summary["tau20000"] = {"gql_steps": gst20["steps"], "model_steps": st20["steps"]}
        # the same graph at tau 5000
        runs = {"gql": [], "model": []}
        for i in range(3):
            _, gst, gkeys = _mine(tfsm, held, 5000, 5, tfsm.ORDER_GQL, None, tmp_path / f"g5_{i}.txt")
            _, mst, mkeys = _mine(tfsm, held, 5000, 5, tfsm.ORDER_MODEL, m, tmp_path / f"m5_{i}.txt")
            assert mkeys == gkeys and len(gkeys) > 100
            runs["gql"].append(gst)
            runs["model"].append(mst)
        gst, mst = (sorted(runs[k], key=lambda r: r["steps"])[1] for k in ("gql", "model"))  # medians
        sample = gkeys[:: max(1, len(gkeys) // 60)]
        mni = {}
        for name, policy in (("gql", tfsm.ORDER_GQL), ("model", tfsm.ORDER_MODEL)):
            with tfsm.Graph.load(held, 5000) as g:
                g.set_order_policy(policy, model=m if policy == tfsm.ORDER_MODEL else None)
                res = g.evaluate([tfsm.parse_key(k) for k in sample], flags=tfsm.FLAG_EXACT)
                mni[name] = [r.mni for r in res]
        assert mni["model"] == mni["gql"]
        gain = gst["steps"] / max(1, mst["steps"])
        summary["tau5000"] = {"patterns": len(gkeys), "gql_steps": [r["steps"] for r in runs["gql"]],
                              "model_steps": [r["steps"] for r in runs["model"]], "median_steps_gain": gain,
                              "gql_search_ms": gst["search_ms"], "model_search_ms": mst["search_ms"]}
        print("learned-order summary:", json.dumps(summary))
        assert gain >= 1.2, summary
    finally:
        m.close()
