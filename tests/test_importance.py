"""Host side of the learned importance: the oracle network's gradients, features,
targets and the roulette-scale transform (no GPU)."""

from __future__ import annotations

import numpy as np
import pytest


def test_oracle_network_gradients_match_finite_differences():
    from oracle import mlp

    rng = np.random.default_rng(1)
    p = mlp.initial(3, 10).astype(np.float64)
    x = rng.normal(size=(7, 10))
    t, w = rng.normal(size=7), rng.uniform(0.5, 1.5, size=7)
    _, g = mlp.gradients(p, x, t, w, bf16_values=False)
    for idx in (0, 5, 16387, 17640, 82178, 83209, mlp.COUNT - 3, mlp.COUNT - 1):
        q = p.copy()
        q[idx] += 1e-6
        up, _ = mlp.gradients(q, x, t, w, bf16_values=False)
        q[idx] -= 2e-6
        down, _ = mlp.gradients(q, x, t, w, bf16_values=False)
        assert g[idx] == pytest.approx((up - down) / 2e-6, rel=1e-5, abs=1e-9)


def test_bf16_rounding_is_nearest_even():
    from oracle import mlp

    assert mlp.bf16(np.float32(1.0 + 2**-8)) == 1.0  # tie to even
    assert mlp.bf16(np.float32(1.0 + 3 * 2**-8)) == 1.0 + 2**-6
    assert mlp.bf16(np.float32(-2.5)) == -2.5


def test_cell_features_cover_every_cell():
    import monki.scenes as scenes
    from monki.importance import FEATURES, cell_features, parse_tables

    scene = scenes.box_cloud(2, 1)
    t = parse_tables(scene.tables)
    f = cell_features(scene.tables)
    assert f.shape == (t.nx * t.ny * t.nz, FEATURES) and np.all(np.isfinite(f))
    # Fortran cell order: the log-extinction feature of cell (i, j, k) is at i + nx (j + ny k).
    i, j, k = 12, 9, 4
    assert f[i + t.nx * (j + t.ny * k), 0] == pytest.approx(np.log10(t.beta[i, j, k] + 1e-6), rel=1e-6)
    assert t.asymmetry[1] == pytest.approx(0.85, abs=0.01)


def test_targets_and_roulette_scale():
    from monki.importance import importance_targets, roulette_scale

    tally = np.zeros((2, 2, 2, 2))
    tally[1] = [[[100, 4], [64, 0]], [[200, 16], [1000, 32]]]
    tally[0] = tally[1] * np.arange(1, 9).reshape(2, 2, 2)
    target, weight = importance_targets(tally, minimum_events=16)
    assert weight[tally[1].ravel(order="F") < 16].max() == 0
    assert weight.max() == 1.0
    scale = roulette_scale(np.log(np.arange(1, 9.0)), (2, 2, 2), exponent=1.0, low=0.25, high=1.0)
    assert scale.shape == (2, 2, 2) and scale.min() >= 0.25 and scale.max() <= 1.0
