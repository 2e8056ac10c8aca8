"""Learned scheduler: features, model file, GPU kernels (gradients checked
against an FP64 CPU forward/backward), and that a learned choice never changes
results."""
import numpy as np
import pytest

import gmr
from gmr import learn as Lr
from helpers import golden_cases, load_case


def small_plan():
    m = gmr.gen_mosaic(2500, 600, 16, 0.02, 0.002, 5, threads=4)
    return gmr.Plan.build(gmr.repair(m, 4), 2500, 600)


def test_features_shape_and_invariants():
    p = small_plan()
    d = p.stats["depth"]
    for sr, B in ((0, 1), (1, 64), (2, 32)):
        f = Lr.launch_features(p, sr, B)
        assert f.shape == (d + 2, Lr.N_BASE)
        assert np.all(f[0] == 0)
        hist = f[1:d + 1, 5:9].sum(axis=1)
        np.testing.assert_allclose(hist, 1.0, atol=1e-6)   # every level has rules
        assert np.all(f[d + 1, 5:9] == 0) and f[d + 1, 0] == 0  # final fold: no rules
        np.testing.assert_allclose(f[1:, 0], np.log1p(p.level_ops()[1:].tolist() + [0]), rtol=1e-6)
        assert f[1, 11] == (sr == 1) and f[1, 12] == (sr == 2)


def test_model_inputs_one_hot():
    base = np.arange(3 * Lr.N_BASE, dtype=np.float32).reshape(3, Lr.N_BASE)
    X = Lr.model_inputs(base).reshape(3, Lr.N_VAR, Lr.IN_DIM)
    assert np.all(X[:, :, :Lr.N_BASE] == base[:, None, :])
    np.testing.assert_array_equal(X[:, :, Lr.N_BASE:], np.broadcast_to(np.eye(Lr.N_VAR), (3, Lr.N_VAR, Lr.N_VAR)))


def test_model_file_round_trip_and_checksum(tmp_path):
    m = Lr.Mlp.create(seed=3)
    assert m.n_params == Lr.IN_DIM * 64 + 64 + 2 * (64 * 64 + 64) + 64 + 1
    m.set_norm(np.linspace(0, 1, Lr.IN_DIM), np.linspace(1, 2, Lr.IN_DIM))
    m.save(tmp_path / "m.gmrmlp")
    m2 = Lr.Mlp.load(tmp_path / "m.gmrmlp")
    np.testing.assert_array_equal(m.params(), m2.params())
    raw = bytearray((tmp_path / "m.gmrmlp").read_bytes())
    raw[100] ^= 0x40
    (tmp_path / "bad.gmrmlp").write_bytes(bytes(raw))
    with pytest.raises(gmr.GmrError) as e:
        Lr.Mlp.load(tmp_path / "bad.gmrmlp")
    assert "checksum" in str(e.value)


def test_committed_model_loads():
    if not Lr.MODEL_PATH.exists():
        pytest.skip("no trained cost model committed")
    m = Lr.Mlp.load(Lr.MODEL_PATH)
    assert m.n_params == Lr.Mlp.create().n_params


# ---------------------------------------------------------------- FP64 reference of the network
def ref_forward_backward(params, mean, std, X, T, hidden=64, layers=3):
    dims = [X.shape[1]] + [hidden] * layers + [1]
    Ws, bs, o = [], [], 0
    for a, b in zip(dims[:-1], dims[1:]):
        Ws.append(params[o:o + a * b].reshape(b, a).astype(np.float64))
        o += a * b
        bs.append(params[o:o + b].astype(np.float64))
        o += b
    A = [(X.astype(np.float64) - mean) / std]
    for i, (W, b) in enumerate(zip(Ws, bs)):
        Z = A[-1] @ W.T + b
        A.append(Z if i == len(Ws) - 1 else np.maximum(Z, 0))
    Y = A[-1][:, 0]
    N = len(X)
    loss = np.mean((Y - T) ** 2)
    dZ = (2 * (Y - T) / N)[:, None]
    grads = [None] * (2 * len(Ws))
    for i in range(len(Ws) - 1, -1, -1):
        grads[2 * i] = dZ.T @ A[i]
        grads[2 * i + 1] = dZ.sum(axis=0)
        if i > 0:
            dZ = (dZ @ Ws[i]) * (A[i] > 0)
    return Y, loss, np.concatenate([g.reshape(-1) for g in grads])


@pytest.mark.gpu
def test_gpu_forward_and_gradients_match_fp64():
    rng = np.random.default_rng(0)
    X = rng.normal(size=(700, Lr.IN_DIM)).astype(np.float32)
    T = rng.normal(size=700).astype(np.float32)
    m = Lr.Mlp.create(seed=5)
    mean, std = X.mean(axis=0), X.std(axis=0)
    m.set_norm(mean, std)
    p = m.params()
    Y64, loss64, g64 = ref_forward_backward(p, mean.astype(np.float64), std.astype(np.float64), X, T)
    Y = m.predict(X)
    np.testing.assert_allclose(Y, Y64, rtol=1e-4, atol=1e-4)
    g, loss = m.gradients(X, T)
    assert abs(loss - loss64) <= 1e-4 * max(1.0, loss64)
    err = np.linalg.norm(g - g64) / np.linalg.norm(g64)
    print(f"gradient rel error vs FP64: {err:.2e}")
    assert err < 1e-4
    # finite differences on a few parameters (FP64 reference), as a check of the reference itself
    for k in rng.choice(len(p), 5, replace=False):
        h = 1e-6  # small enough that no ReLU input changes sign
        pp, pm = p.astype(np.float64).copy(), p.astype(np.float64).copy()
        pp[k] += h
        pm[k] -= h
        lp = ref_forward_backward(pp, mean, std, X, T)[1]
        lm = ref_forward_backward(pm, mean, std, X, T)[1]
        assert abs((lp - lm) / (2 * h) - g64[k]) < 1e-7 + 1e-4 * abs(g64[k])


@pytest.mark.gpu
def test_gpu_training_fits_a_function():
    rng = np.random.default_rng(1)
    X = rng.normal(size=(4096, Lr.IN_DIM)).astype(np.float32)
    T = (np.sin(X[:, 0]) + 0.5 * X[:, 1] * X[:, 2] + X[:, 20]).astype(np.float32)
    m = Lr.Mlp.create(seed=2)
    m.set_norm(np.zeros(Lr.IN_DIM), np.ones(Lr.IN_DIM))
    before = float(np.mean((m.predict(X) - T) ** 2))
    after = m.train(X, T, epochs=40, batch=256, lr=3e-3, seed=4)
    print(f"train MSE {before:.3f} -> {after:.4f}")
    assert after < 0.1 * before


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_cases()[:2])
def test_learned_choice_keeps_results(name):
    torch = pytest.importorskip("torch")
    c = load_case(name)
    g = gmr.Grammar.from_arrays(int(c["alpha"]), c["rules"], c["C"], c["V"])
    plan = gmr.Plan.build(g, int(c["rows"]), int(c["cols"]))
    eng = gmr.Engine(plan)
    rng = np.random.default_rng(0)
    X = rng.uniform(-1, 1, (int(c["cols"]), 32)).astype(np.float32)
    ref = eng.multiply(X, 0, B=32, variant=gmr.VARIANT_PLAIN)
    m = Lr.Mlp.load(Lr.MODEL_PATH) if Lr.MODEL_PATH.exists() else Lr.Mlp.create(seed=9)
    pred = Lr.choose_learned(eng, plan, m, 0, 32)
    table = eng.level_variants(0, 32)
    assert table is not None and np.array_equal(table[1:], pred[1:].argmin(axis=1))
    Y = eng.multiply(X, 0, B=32)  # AUTO: the learned table
    np.testing.assert_allclose(Y, ref, rtol=1e-5, atol=1e-5)


def test_mode_chain_recursion_matches_brute_force():
    """best_chain (the mode model's choice of pull / interleave per level)
    finds the cheapest chain that exhaustive enumeration finds, with levels
    that cannot interleave and unmeasured pairs respected."""
    import itertools

    rng = np.random.default_rng(4)
    for trial in range(40):
        n = int(rng.integers(3, 9))  # slots: prologue, levels 1..n-2, final fold
        cost = rng.uniform(1.0, 10.0, (n, 3, 3))
        allowed = rng.random(n) < 0.6
        allowed[0] = allowed[-1] = False
        if trial % 3 == 0:
            cost[rng.integers(1, n), Lr.INTERLEAVE, Lr.PULL] = np.nan  # a pair never measured
        modes, total = Lr.best_chain(cost, allowed)
        best = np.inf
        for combo in itertools.product((Lr.PULL, Lr.INTERLEAVE), repeat=n - 2):
            ms = [Lr.PULL, *combo, Lr.PULL]
            if any(m == Lr.INTERLEAVE and not allowed[k] for k, m in enumerate(ms)):
                continue
            t = sum(cost[k][ms[k - 1]][ms[k]] for k in range(1, n))
            if np.isfinite(t):
                best = min(best, t)
        assert np.isclose(total, best)
        assert np.isclose(sum(cost[k][modes[k - 1]][modes[k]] for k in range(1, n)), total)
        assert all(m == Lr.PULL or allowed[k] for k, m in enumerate(modes))


def test_mode_rows_use_measured_pairs_only():
    base = np.arange(4 * Lr.N_BASE, dtype=np.float32).reshape(4, Lr.N_BASE)
    costs = np.full((4, 3, 3), -1.0, np.float32)
    costs[1, Lr.PULL, Lr.PULL] = 0.5
    costs[2, Lr.PULL, Lr.INTERLEAVE] = 2.0
    costs[3, Lr.INTERLEAVE, Lr.PULL] = 1.0
    costs[0, Lr.PULL, Lr.PULL] = 9.0  # the prologue slot is never a training row
    X, T = Lr.mode_rows(base, costs)
    assert X.shape == (3, Lr.MODE_IN)
    got = {(tuple(x[Lr.N_BASE:]), float(x[0])): t for x, t in zip(X, T)}
    assert np.isclose(got[((0.0, 0.0), float(base[1, 0]))], np.log(500.0))
    assert np.isclose(got[((0.0, 1.0), float(base[2, 0]))], np.log(2000.0))
    assert np.isclose(got[((1.0, 0.0), float(base[3, 0]))], np.log(1000.0))
