"""Many scenes of uneven size on one GB300.

``run_persistent`` (the default of ``run_batched``) runs every scene in one launch sequence:
the scenes share one photon pool, each wavefront launch covers all of them (thread blocks
serve one scene each; see csrc/multi.cu), and each batch of iterations replays as a CUDA
graph. ``run_batched(..., persistent=False)`` instead gives each scene its own resident
session (own stream) and drives up to ``concurrency`` of them from host threads, with
launch shapes from the autotuner per scene.

Either way each scene's result is exactly what running the scene alone gives (its own
random streams, keyed by its photons, rounds and seed).
"""

from __future__ import annotations

import ctypes
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from .execution import CUDA, BatchControls
from .execution import native as _native
from .execution.tallies import RawTallies


def run_scene(scene, *, device: int = 0, seed: int = 23274, rounds: int = 1, options=None):
    options = options or {}
    with CUDA(device=device, seed=seed, **options) as backend:
        backend.prepare(scene)
        batches = backend.run_batches([BatchControls(i, scene.photons_per_column) for i in range(1, rounds + 1)])
        return batches, dict(backend.provenance)


def run_persistent(scenes, *, device: int = 0, seed: int = 23274, rounds: int = 1, precision: str = "fp32",
                   pool: int = 1 << 22, walk: int = 2, check_every: int = 8, graphs: bool = True,
                   max_steps: int = 100_000, tail: int = 1 << 16, library=None):
    """Every scene in one multi-scene session: returns (per-scene (batches, provenance),
    summary). Scenes are forward, without layer paths, with I or I/Q/U."""

    if not scenes:
        raise ValueError("no scenes")
    if precision not in ("fp32", "fp64"):
        raise ValueError("precision must be 'fp32' or 'fp64'")
    native = _native.load(library) if library else _native.load()
    tables = [np.ascontiguousarray(s.tables, dtype=np.float64) for s in scenes]
    n = len(tables)
    pointers = (_native.F64P * n)(*[t.ctypes.data_as(_native.F64P) for t in tables])
    counts = (ctypes.c_size_t * n)(*[t.size for t in tables])
    config = (f"precision={precision},pool={pool},walk={walk},check_every={check_every},graphs={int(graphs)},"
              f"tail={int(tail)}")
    error = ctypes.create_string_buffer(8192)
    handle = native.monki_cuda_multi_create(device, n, pointers, counts, rounds, config.encode(), error, len(error))
    if not handle:
        raise RuntimeError(error.value.decode())
    try:
        controls = np.zeros((n, 8), dtype=np.uint32)
        outputs = []
        for q, scene in enumerate(scenes):
            nmat, nx, ny, nz, angles = scene.shape
            per_round = scene.photons_per_column * nx * ny
            controls[q] = [per_round * rounds, 0, 1, seed, max_steps, 0, per_round, rounds]
            outputs.append(np.zeros(rounds * int(native.monki_cuda_multi_tally_count(handle, q))))
        out = (_native.F64P * n)(*[o.ctypes.data_as(_native.F64P) for o in outputs])
        start = time.perf_counter()
        if native.monki_cuda_multi_run(handle, controls.ctypes.data_as(_native.U32P), out, error, len(error)):
            raise RuntimeError(error.value.decode())
        wall = time.perf_counter() - start
        totals = (ctypes.c_uint64 * 6)()
        timing = (ctypes.c_float * 2)()
        native.monki_cuda_multi_counters(handle, totals)
        native.monki_cuda_multi_last_timing(handle, timing)
        per_scene = []
        for q in range(n):
            counts = (ctypes.c_uint64 * 6)()
            native.monki_cuda_multi_scene_counters(handle, q, counts)
            per_scene.append([int(v) for v in counts])
    finally:
        native.monki_cuda_multi_close(handle)
    results = []
    for scene, values, counts in zip(scenes, outputs, per_scene, strict=True):
        nmat, nx, ny, nz, angles = scene.shape
        per = values.reshape(rounds, -1)
        batches = [RawTallies(BatchControls(r + 1, scene.photons_per_column),
                              per[r].reshape((nmat, nx, ny, angles), order="F").copy()) for r in range(rounds)]
        results.append((batches, {"backend": "cuda-multi-scene", "precision": precision, "seed": seed,
                                  "scatters": counts[0], "photons": counts[4], "tail_launches": counts[5]}))
    summary = {"scenes": n, "wall_s": wall, "device_s": timing[1] / 1e3, "scatters": int(totals[0]),
               "photons": int(totals[4]), "scatters_per_s": totals[0] / wall,
               "device_scatters_per_s": totals[0] / max(timing[1] / 1e3, 1e-9), "kernel_launches": int(totals[5]),
               "tails": sum(c[5] for c in per_scene), "persistent": True, "pool": pool}
    return results, summary


def run_batched(scenes, *, device: int = 0, seed: int = 23274, rounds: int = 1, concurrency: int = 4, tune=None,
                persistent: bool = True, **options):
    """Run every scene; returns (per-scene (batches, provenance), summary). With
    ``persistent`` (default) all scenes share one multi-scene launch sequence
    (``run_persistent``, keyword options pass through); otherwise each scene gets its own
    session, ``tune`` mapping a scene to CUDA launch options (for example
    ``lambda s: autotune(s).options()``), up to ``concurrency`` at a time."""

    if persistent:
        return run_persistent(scenes, device=device, seed=seed, rounds=rounds, **options)
    settings = [tune(scene) if tune else {} for scene in scenes]
    start = time.perf_counter()
    with ThreadPoolExecutor(max_workers=max(1, concurrency)) as pool:
        futures = [pool.submit(run_scene, scene, device=device, seed=seed, rounds=rounds, options=o)
                   for scene, o in zip(scenes, settings, strict=True)]
        results = [f.result() for f in futures]
    wall = time.perf_counter() - start
    scatters = sum(p["scatters"] for _, p in results)
    photons = sum(p["photons"] for _, p in results)
    return results, {"scenes": len(scenes), "wall_s": wall, "scatters": scatters, "photons": photons,
                     "scatters_per_s": scatters / wall, "concurrency": concurrency, "persistent": False}


def main(argv=None) -> int:
    """``python -m monki.batched``: the batched workload's seeded scenes (``batched_scene``)
    in one multi-scene session; prints the run's summary."""

    import argparse
    import json

    from .scenes import batched_scene

    parser = argparse.ArgumentParser(prog="python -m monki.batched")
    parser.add_argument("--scenes", type=int, default=64)
    parser.add_argument("--photons-scale", type=float, default=0.05)
    parser.add_argument("--rounds", type=int, default=1)
    parser.add_argument("--precision", choices=("fp32", "fp64"), default="fp32")
    parser.add_argument("--device", type=int, default=0)
    args = parser.parse_args(argv)
    batch = [batched_scene(seed, photons_scale=args.photons_scale) for seed in range(args.scenes)]
    _, summary = run_persistent(batch, device=args.device, rounds=args.rounds, precision=args.precision)
    print(json.dumps(summary))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
