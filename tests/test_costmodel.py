"""The learned matching-order cost model (a 32-64-64-1 MLP with BF16 weights, trained on the GPU).

CPU: the numpy oracle's backpropagation equals central finite differences (without BF16 rounding).
GPU: the hand-written kernels' predictions and gradients equal the oracle's (same BF16 rounding
points; FP32 vs float64 sums and the order of atomic adds are the only differences, hence the
tolerances); Adam training lowers the loss; and a model trained on records logged by the plain
miner chooses orders that leave the mined pattern set and every exact MNI support unchanged.
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


def _gen(built, out, seed, n):
    import subprocess

    subprocess.run([str(built / "bin" / "gen_lg"), "--out", str(out), "--n", str(n), "--mean", "22", "--gamma", "2.2",
                    "--max-degree", "1400", "--labels", "29", "--zipf", "1.2", "--elabels", "1", "--seed", str(seed)],
                   check=True, capture_output=True)
    return out


@pytest.mark.gpu
def test_learned_orders_keep_results_and_report_gain(tfsm, built, tmp_path):
    """Records from the plain miner with random orders (training graphs, seeds 10-13) train the
    model; on a held-out graph (seed 99) the model's orders give the same pattern set and the
    same exact MNI supports as the fixed GQL order.  The steps of both are written to the log."""
    import json

    n, tau, max_nodes = 30000, 2700, 5
    feats, costs = [], []
    for seed in (10, 11, 12, 13):
        with tfsm.Graph.load(_gen(built, tmp_path / f"train{seed}.lg", seed, n), tau) as g:
            g.set_order_policy(tfsm.ORDER_RANDOM, seed=seed)
            g.record_orders(True)
            g.mine(max_nodes=max_nodes, flags=tfsm.FLAG_PLAIN)
            f, c = g.take_records()
            feats.append(f)
            costs.append(c)
    x, t = np.concatenate(feats), np.concatenate(costs)
    assert len(x) >= 200, len(x)
    m = tfsm.CostModel(seed=5)
    try:
        mse0 = mlp_oracle.loss(m.params(), x, t)
        mse = m.train(x, t, epochs=60, batch=64, lr=2e-3, seed=3)
        assert mse < mse0
        held = _gen(built, tmp_path / "held99.lg", 99, n)
        out = {}
        for name, policy in (("gql", tfsm.ORDER_GQL), ("model", tfsm.ORDER_MODEL)):
            with tfsm.Graph.load(held, tau) as g:
                g.set_order_policy(policy, model=m if policy == tfsm.ORDER_MODEL else None)
                path = tmp_path / f"{name}.txt"
                st = g.mine(max_nodes=max_nodes, results_path=path)
                pats = tfsm.read_results(path)
                keys = sorted(set(pats))
                exact = g.evaluate([tfsm.parse_key(k) for k in keys], flags=tfsm.FLAG_EXACT)
                out[name] = dict(patterns=keys, mni={k: r.mni for k, r in zip(keys, exact)}, steps=st["steps"],
                                 search_ms=st["search_ms"], evaluations=st["evaluations"])
                # records of the held-out run: how well does the model rank orders it never saw?
        assert out["model"]["patterns"] == out["gql"]["patterns"]
        assert out["model"]["mni"] == out["gql"]["mni"]
        summary = {k: {kk: v[kk] for kk in ("steps", "search_ms", "evaluations")} for k, v in out.items()}
        summary["records"] = int(len(x))
        summary["train_mse"] = [mse0, mse]
        summary["steps_gain"] = out["gql"]["steps"] / max(1, out["model"]["steps"])
        print("learned-order summary:", json.dumps(summary))
    finally:
        m.close()
