"""What the trained cost model gains: on a grammar the committed model never
saw (held out of its corpus), the learned per-launch tables are compared with
the engine's untuned default and with the exhaustive autotuner.

* Gain: the summed CUDA-graph multiply time of the learned tables over six
  (semiring, B) cases is not above the default's (beyond 3 % of noise).
* Regret: on the autotuner's own per-launch measurements, the learned picks
  cost at most 10 % more than the measured best on average over the cases
  (the bar of the learned scheduler), and no case more than 25 % (the
  measurements of one small grammar's short launches carry a few % of
  noise, so a per-case 10 % bar would flake).
"""
import numpy as np
import pytest

import gmr
from gmr import learn

HELD_OUT = 54  # corpus grammar index: a 98,160 x 7,210 mosaic (seed 154)
CASES = [(0, 8), (0, 32), (1, 32), (1, 128), (2, 8), (2, 32)]


def held_out_indices(n_mosaic=192, n_graph=64, holdout=0.25):
    """The split gmr.learn uses: a seeded permutation of the corpus."""
    n = n_mosaic + n_graph
    order = np.random.default_rng(7).permutation(n)
    return set(order[: int(round(n * holdout))].tolist())


def test_held_out_grammar_is_held_out():
    assert HELD_OUT in held_out_indices()
    spec = learn.corpus_specs(192, 64)[HELD_OUT]
    assert spec["kind"] == "mosaic" and spec["seed"] == 154


@pytest.fixture(scope="module")
def engine():
    pytest.importorskip("torch")
    if not learn.MODEL_PATH.exists():
        pytest.fail("the trained cost model is missing: " + str(learn.MODEL_PATH))
    spec = learn.corpus_specs(192, 64)[HELD_OUT]
    g, rows, cols = learn.make_grammar(spec, device=0)
    plan = gmr.Plan.build(g, rows, cols, device=0)
    return gmr.Engine(plan), plan, learn.Mlp.load(learn.MODEL_PATH)


@pytest.mark.gpu
def test_learned_tables_gain_over_default_and_regret(engine):
    eng, plan, model = engine
    t_default = t_learned = 0.0
    regrets = {}
    for sr, B in CASES:
        seed = 10 * sr + B
        d = min(learn.sweep_time(eng, sr, B, None, seed, n=20) for _ in range(3))
        mode_model = learn.Mlp.load(learn.MODE_MODEL_PATH) if learn.MODE_MODEL_PATH.exists() else None
        pred = learn.choose_learned(eng, plan, model, sr, B, mode_model=mode_model)
        table = eng.level_variants(sr, B)
        lt = min(learn.sweep_time(eng, sr, B, table, seed, n=20) for _ in range(3))
        t_default += d
        t_learned += lt
        # regret on the autotuner's own measurements (launch slots 1.., 20 variants)
        import torch

        X, words = learn.random_inputs(torch, sr, eng.cols, B, seed)
        Y = torch.empty((eng.rows, words), device="cuda", dtype=X.dtype)
        times = eng.autotune(sr, X.data_ptr(), Y.data_ptr(), B, stream=torch.cuda.current_stream().cuda_stream)[1:]
        pick = pred[1:].argmin(axis=1)
        regrets[(sr, B)] = times[np.arange(len(pick)), pick].sum() / times.min(axis=1).sum() - 1.0
    print(f"learned {t_learned:.3f} ms, default {t_default:.3f} ms, gain {t_default / t_learned:.3f}x; "
          f"regret per case {regrets}")
    assert t_learned <= 1.03 * t_default, (t_learned, t_default)
    assert float(np.mean(list(regrets.values()))) <= 0.10, regrets
    assert max(regrets.values()) <= 0.25, regrets
