"""CPU checks of the warm-start network's oracle (oracle/nn_oracle.py) and of
the seeded random decks: the oracle's backward pass against central finite
differences in FP64, and the decks' determinism and validity."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import nn_oracle as nn  # noqa: E402

import tealeaf_cuda_gb300 as tl  # noqa: E402
from tealeaf_cuda_gb300 import learned  # noqa: E402


def _loss(params, x, t, margin):
    y, _ = nn.forward(params, x, quant=False)
    return nn.loss_and_dy(y, t, margin, quant=False)[0]


def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    params = learned.init_params(3, head_scale=1.0).astype(np.float64)
    B, H, W, margin = 1, 12, 12, 2
    x = np.zeros((B, H + 2, W + 2, 16))
    x[:, 1:-1, 1:-1, :5] = rng.normal(0, 1, (B, H, W, 5))
    t = rng.normal(0, 0.1, (B, H, W))
    y, cache = nn.forward(params, x, quant=False)
    _, dy = nn.loss_and_dy(y, t, margin, quant=False)
    grads = nn.backward(params, cache, dy, quant=False)
    flat = np.concatenate([np.concatenate([dw.ravel(), db]) for dw, db in grads])
    assert flat.size == params.size
    # layer boundaries, so every layer's weights and biases are probed
    idx = []
    off = 0
    for cin, co, _ in nn.LAYERS:
        nw = 9 * co * cin
        live = [k for k in range(off, off + nw) if (k - off) % cin < (5 if off == 0 else cin)]
        idx += list(rng.choice(live, 3, replace=False)) + [off + nw]
        off += nw + co
    h = 1e-6
    for k in idx:
        p1, p2 = params.copy(), params.copy()
        p1[k] += h
        p2[k] -= h
        fd = (_loss(p1, x, t, margin) - _loss(p2, x, t, margin)) / (2 * h)
        assert flat[k] == pytest.approx(fd, rel=1e-4, abs=1e-9), k


def test_bf16_rounding_is_round_to_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, -2.5, 3.0e-3], dtype=np.float64)
    r = nn.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0078125
    assert r[3] == -2.5
    assert abs(r[4] - 3.0e-3) < 3.0e-3 * 2 ** -8


def test_random_decks_are_seeded_and_parse():
    a, b, c = learned.random_deck(7, 64, 3), learned.random_deck(7, 64, 3), learned.random_deck(8, 64, 3)
    assert a == b and a != c
    for s in range(20):
        states = learned.random_states(s)
        assert 4 <= len(states) <= 9
        for st in states:
            assert 0.05 <= st["density"] <= 200.0
            assert 1e-4 <= st["energy"] <= 50.0
        cfg = tl.parse_deck(learned.random_deck(s, 64, 3))
        assert cfg.nstates == len(states) and cfg.x_cells == 64


def test_model_file_round_trip(tmp_path):
    p = learned.init_params(5)
    f = tmp_path / "m.tlws"
    learned.save_model(str(f), p)
    q = learned.load_model(str(f))
    assert np.array_equal(p, q)
    assert q.size == learned.param_count() == tl.load().tl_warm_start_param_count()
