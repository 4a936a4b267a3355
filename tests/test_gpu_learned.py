"""The trained importance network on held-out box clouds.

The network is trained on the device from analog-kernel importance tallies of the
training family (batched-generator scenes and randomly placed box clouds) and applied to
box clouds it has not seen. Checked: its prediction explains the held-out pilot tallies
(weighted R^2), the guided estimate with the learned roulette map agrees with the analog
kernel within combined standard error (the map moves variance, never the expectation),
and what the network gains over guided transport without it: variance x time of the
median pixel improves (the worst pixel does not; the time to a precision target in every
pixel is set by constant roulette).
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rounds(scene, guided, scale, ppc, rounds, seed):
    import time

    from monki.execution import CUDA, BatchControls

    with CUDA(guided=guided, seed=seed, roulette_scale=scale) as backend:
        backend.prepare(scene)
        start = time.perf_counter()
        batches = backend.run_batches([BatchControls(i, ppc) for i in range(1, rounds + 1)])
        elapsed = time.perf_counter() - start
    return np.stack([b.stokes[0] for b in batches]) / ppc, elapsed


def test_learned_importance_generalises_and_keeps_estimates_unbiased(device):
    import monki.scenes as scenes
    from monki import Guided
    from monki.importance import (cell_features, importance_targets, learned_scale, pilot, r_squared,
                                  train_model, training_scenes)

    model, losses, rows = train_model(training_scenes(6), steps=600, batch=8192, rows_per_scene=8000)
    with model:
        assert np.all(np.isfinite(losses)) and losses[-50:].mean() < 0.5 * losses[:20].mean()
        gains = []
        for seed in (1000, 1001):
            # 64 rounds: roulette makes the estimates skewed, and with few rounds a low sample
            # mean comes with a low sample variance, which pulls the mean z below zero.
            scene = scenes.box_cloud_variant(seed, 2000, 64)
            tally, _ = pilot(scene, rounds=2, photons_per_column=300, seed=3)
            target, weight = importance_targets(tally)
            prediction = model.predict(cell_features(scene.tables))
            assert r_squared(prediction[weight > 0], target[weight > 0], weight[weight > 0]) > 0.8
            scale = learned_scale(model, scene)
            plain, t_plain = _rounds(scene, None, None, 2000, 64, seed)
            constant, t_constant = _rounds(scene, Guided(0.0, 1.0, 0.0), None, 2000, 64, seed + 1)
            learned, t_learned = _rounds(scene, Guided(0.0, 1.0, 0.0), scale, 2000, 64, seed + 2)
            n = plain.shape[0]
            se = lambda a: a.std(0, ddof=1) / np.sqrt(n)  # noqa: E731
            z = (learned.mean(0) - plain.mean(0)) / np.hypot(se(learned), se(plain))
            assert np.mean(np.abs(z) < 3) >= 0.99 and abs(z.mean()) < 0.1
            relative = lambda a: np.median(se(a) / np.abs(a.mean(0)))  # noqa: E731
            merit = lambda a, t: 1.0 / (relative(a) ** 2 * t)  # noqa: E731
            gains.append(merit(learned, t_learned) / merit(constant, t_constant))
        print(f"learned roulette map: median-pixel variance x time gain over constant roulette {gains}")
        assert np.mean(gains) > 1.0
