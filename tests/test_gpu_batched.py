"""CUDA-graph replay, batched scenes and the autotuner on the GB300.

* a round group replayed as CUDA graphs gives the tallies of the same group launched
  kernel by kernel (FP64 transport; only the device's atomic summation order differs);
* scenes of uneven size in one multi-scene launch sequence (one shared photon pool, every
  launch covering all scenes) give each scene exactly what running it alone gives, with
  and without graph replay, I and I/Q/U scenes together;
* scenes of uneven size run concurrently from host threads in their own sessions do too;
* the autotuner times its candidates and returns the fastest.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _flat(batches):
    return np.concatenate([b.stokes.ravel(order="F") for b in batches])


def test_graph_replay_equals_kernel_launches(native, device):
    import monki.scenes as scenes
    from monki.execution.native import F64P

    scene = scenes.box_cloud(20, 2, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))
    tables = np.ascontiguousarray(scene.tables)
    per_round = 20 * 120
    results = []
    for graphs in (1, 0):
        err = ctypes.create_string_buffer(1024)
        handle = native.monki_cuda_create(0, tables.ctypes.data_as(F64P), tables.size, 2,
                                          f"precision=fp64,pool=1024,graphs={graphs}".encode(), err, len(err))
        assert handle, err.value
        out = np.zeros(2 * native.monki_cuda_tally_count(handle))
        controls = (ctypes.c_uint32 * 8)(2 * per_round, 0, 1, 9, 100000, 0, per_round, 2)
        assert native.monki_cuda_run(handle, controls, out.ctypes.data_as(F64P), err, len(err)) == 0, err.value
        native.monki_cuda_close(handle)
        results.append(out)
    np.testing.assert_allclose(results[0], results[1], rtol=1e-9, atol=1e-15)


def test_batched_scenes_equal_scenes_run_alone(device):
    import monki.scenes as scenes
    from monki.batched import run_batched, run_scene

    batch = [scenes.batched_scene(seed, photons_scale=0.002) for seed in range(4)]
    results, summary = run_batched(batch, concurrency=4, tune=lambda s: {"precision": "fp64"}, persistent=False)
    assert summary["scenes"] == 4 and summary["scatters"] > 0
    for scene, (batches, provenance) in zip(batch, results, strict=True):
        alone, alone_provenance = run_scene(scene, options={"precision": "fp64"})
        assert provenance["scatters"] == alone_provenance["scatters"]
        np.testing.assert_allclose(_flat(batches), _flat(alone), rtol=1e-9, atol=1e-15)


def _persistent_batch():
    import monki.scenes as scenes

    batch = [scenes.batched_scene(seed, photons_scale=0.002) for seed in (0, 1, 2, 5, 11, 17)]
    batch.append(scenes.batched_scene(93, photons_scale=0.0005, grid=(128, 128)))
    assert {s.shape[0] for s in batch} == {1, 3}
    return batch


@pytest.mark.parametrize("graphs", [True, False])
def test_persistent_scenes_equal_scenes_run_alone(device, graphs):
    """Seven uneven scenes (grids 8-128 columns a side, I and I/Q/U, 20-60 layers) in one
    multi-scene session, FP64, two rounds each, wavefront launches to the end (no tail
    kernel): every scene's tallies and scatter count equal the scene run alone in its own
    session (same seed)."""

    from monki.batched import run_persistent, run_scene

    batch = _persistent_batch()
    results, summary = run_persistent(batch, rounds=2, precision="fp64", pool=1 << 18, graphs=graphs, tail=0)
    assert summary["scenes"] == len(batch) and summary["scatters"] > 0
    scatters = 0
    for scene, (batches, provenance) in zip(batch, results, strict=True):
        alone, alone_provenance = run_scene(scene, rounds=2, options={"precision": "fp64", "tail": 0})
        assert provenance["scatters"] == alone_provenance["scatters"]
        scatters += alone_provenance["scatters"]
        np.testing.assert_allclose(_flat(batches), _flat(alone), rtol=1e-9, atol=1e-15)
    assert summary["scatters"] == scatters


def test_persistent_tail_launches_match_scenes_run_alone(device):
    """The same scenes with tail launches (each scene's last photons in its own launch, once
    the group's photons are all claimed). The tail kernel inlines the same slot functions
    as the wavefront kernels, but the compiler contracts their arithmetic differently, and a
    scene's tail starts at another iteration than when it runs alone, so a few FP64
    histories of a large scene part ways after a rounding-level difference. Checked: tails
    ran, every scene's scatter count is within 0.2 % of the scene run alone, and its
    domain-summed Stokes I within 0.5 % (the test above pins the launches themselves)."""

    from monki.batched import run_persistent, run_scene

    batch = _persistent_batch()
    results, summary = run_persistent(batch, rounds=2, precision="fp64", pool=1 << 18, tail=1 << 12)
    assert summary["tails"] > 0, summary
    for q, (scene, (batches, provenance)) in enumerate(zip(batch, results, strict=True)):
        alone, alone_provenance = run_scene(scene, rounds=2, options={"precision": "fp64", "tail": 1 << 12})
        detail = (q, provenance["scatters"], alone_provenance["scatters"], provenance["tail_launches"])
        assert abs(provenance["scatters"] / alone_provenance["scatters"] - 1.0) < 2e-3, detail
        total = sum(float(b.stokes[0].sum()) for b in batches)
        total_alone = sum(float(b.stokes[0].sum()) for b in alone)
        assert abs(total / total_alone - 1.0) < 5e-3, (detail, total, total_alone)


def test_persistent_fp32_scenes_agree_with_scenes_run_alone(device):
    """The FP32 product path of the multi-scene session (wavefront launches to the end in
    both) against the scenes run alone. The multi-scene and single-scene kernels inline the
    same slot functions in different kernels, and with the fast FP32 math of the transport
    build a rounding-level difference now and then sends a history another way, so: every
    scene's scatter count within 0.05 % of the scene run alone, and all but 0.1 % of its
    tally entries equal to FP32 summation order (the FP64 test above pins the launches)."""

    import monki.scenes as scenes
    from monki.batched import run_persistent, run_scene

    batch = [scenes.batched_scene(seed, photons_scale=0.01) for seed in (3, 4, 6, 7)]
    results, summary = run_persistent(batch, rounds=1, tail=0)
    for scene, (batches, provenance) in zip(batch, results, strict=True):
        alone, alone_provenance = run_scene(scene, options={"tail": 0})
        assert abs(provenance["scatters"] / alone_provenance["scatters"] - 1.0) < 5e-4
        a, b = _flat(batches), _flat(alone)
        close = np.isclose(a, b, rtol=2e-4, atol=1e-7 * np.abs(b).max())
        assert np.mean(close) >= 0.999, (np.mean(close), np.max(np.abs(a - b)))


def test_sessions_open_and_close_while_others_replay_graphs(device):
    """Sixteen uneven scenes on four host threads, CUDA graphs on and launch shapes from the
    autotuner: sessions are created and destroyed (device allocations and frees) while the
    other threads build and replay their graphs. Every scene still gives exactly what it
    gives run alone."""

    import monki.scenes as scenes
    from monki.batched import run_batched, run_scene
    from monki.tuning import autotune

    batch = [scenes.batched_scene(seed, photons_scale=0.003) for seed in range(16)]
    shapes = {}

    def tune(scene):
        _, nx, ny, _, _ = scene.shape
        key = nx * ny * scene.photons_per_column >= 1 << 16
        if key not in shapes:
            shapes[key] = autotune(scene, device=0, photons_per_round=1 << 16).options()
        return {**shapes[key], "precision": "fp64"}

    for attempt in range(2):
        results, summary = run_batched(batch, concurrency=4, tune=tune, persistent=False)
        assert summary["scenes"] == 16 and summary["scatters"] > 0
        for scene, (batches, provenance) in zip(batch, results, strict=True):
            alone, alone_provenance = run_scene(scene, options=tune(scene))
            assert provenance["scatters"] == alone_provenance["scatters"], (attempt, scene.description)
            np.testing.assert_allclose(_flat(batches), _flat(alone), rtol=1e-9, atol=1e-15)


def test_autotuner_returns_the_fastest_candidate(device):
    import monki.scenes as scenes
    from monki.tuning import autotune

    tuned = autotune(scenes.box_cloud(500, 1), photons_per_round=300_000)
    rates = [rate for _, rate in tuned.trials]
    assert tuned.scatters_per_second == max(rates) > 0
    assert set(tuned.options()) == {"pool", "block", "walk"}
