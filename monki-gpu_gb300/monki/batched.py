"""Many scenes of uneven size on one GB300.

Each scene gets its own resident session (tables, photon pool, tallies on its own CUDA
stream) with the launch shape the autotuner chose for its shape; host threads drive up to
``concurrency`` sessions at once, so the device overlaps the kernels of small scenes that
would not fill it alone. Results are per scene, exactly what running the scene alone gives
(independent sessions, the same seeds).
"""

from __future__ import annotations

import time
from concurrent.futures import ThreadPoolExecutor

from .execution import CUDA, BatchControls


def run_scene(scene, *, device: int = 0, seed: int = 23274, rounds: int = 1, options=None):
    options = options or {}
    with CUDA(device=device, seed=seed, **options) as backend:
        backend.prepare(scene)
        batches = backend.run_batches([BatchControls(i, scene.photons_per_column) for i in range(1, rounds + 1)])
        return batches, dict(backend.provenance)


def run_batched(scenes, *, device: int = 0, seed: int = 23274, rounds: int = 1, concurrency: int = 4, tune=None):
    """Run every scene; returns (per-scene (batches, provenance), summary). ``tune`` maps a
    scene to CUDA launch options (for example ``lambda s: autotune(s).options()``)."""

    options = [tune(scene) if tune else {} for scene in scenes]
    start = time.perf_counter()
    with ThreadPoolExecutor(max_workers=max(1, concurrency)) as pool:
        futures = [pool.submit(run_scene, scene, device=device, seed=seed, rounds=rounds, options=o)
                   for scene, o in zip(scenes, options, strict=True)]
        results = [f.result() for f in futures]
    wall = time.perf_counter() - start
    scatters = sum(p["scatters"] for _, p in results)
    photons = sum(p["photons"] for _, p in results)
    return results, {"scenes": len(scenes), "wall_s": wall, "scatters": scatters, "photons": photons,
                     "scatters_per_s": scatters / wall, "concurrency": concurrency}
