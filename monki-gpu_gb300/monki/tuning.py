"""Launch-shape autotuner for the wavefront transport.

The photon-pool size, the thread-block size and the per-launch walk budget trade
occupancy, queue length and divergence differently for each scene (grid, layer count,
cloud cover, photons per round). ``autotune`` times one short round of the scene under
each candidate on the device (CUDA events around the round group, no host copies in the
timing) and returns the fastest, in scatters per second. Results are cached per scene
shape and photons per round, so a batch of similar scenes tunes once.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from .execution import native as _native

CANDIDATES = (
    {"pool": 1 << 22, "block": 256, "walk": 3},
    {"pool": 1 << 22, "block": 256, "walk": 2},
    {"pool": 1 << 20, "block": 256, "walk": 3},
    {"pool": 1 << 20, "block": 128, "walk": 3},
    {"pool": 1 << 19, "block": 256, "walk": 2},
    {"pool": 1 << 21, "block": 256, "walk": 3},
    {"pool": 1 << 18, "block": 128, "walk": 2},
    {"pool": 1 << 22, "block": 256, "walk": 24},
)


@dataclass(frozen=True)
class Tuned:
    pool: int
    block: int
    walk: int
    scatters_per_second: float
    trials: tuple

    def options(self) -> dict:
        """Keyword arguments of ``monki.execution.CUDA``."""

        return {"pool": self.pool, "block": self.block, "walk": self.walk}


_cache: dict = {}


def _time(native, tables, device, config, per_round, seed):
    error = ctypes.create_string_buffer(4096)
    handle = native.monki_cuda_create(device, tables.ctypes.data_as(_native.F64P), tables.size, 1,
                                      config.encode(), error, len(error))
    if not handle:
        raise RuntimeError(error.value.decode())
    try:
        out = np.zeros(int(native.monki_cuda_tally_count(handle)))
        timing = (ctypes.c_float * 2)()
        counters = (ctypes.c_uint64 * 6)()
        rates = []
        for attempt in range(2):  # the first round warms the session up
            before = (ctypes.c_uint64 * 6)()
            native.monki_cuda_counters(handle, before)
            controls = (ctypes.c_uint32 * 8)(per_round, 0, 900001 + attempt, seed, 100000, 0, per_round, 1)
            if native.monki_cuda_run(handle, controls, out.ctypes.data_as(_native.F64P), error, len(error)):
                raise RuntimeError(error.value.decode())
            native.monki_cuda_last_timing(handle, timing)
            native.monki_cuda_counters(handle, counters)
            rates.append((counters[0] - before[0]) / max(timing[1], 1e-6) * 1e3)
        return rates[-1]
    finally:
        native.monki_cuda_close(handle)


def autotune(scene, *, device: int = 0, photons_per_round: int | None = None, candidates=CANDIDATES,
             precision: str = "fp32", seed: int = 4242) -> Tuned:
    """The fastest candidate launch shape for one short round of the scene."""

    nmat, nx, ny, nz, angles = scene.shape
    per_round = photons_per_round or min(scene.photons_per_column * nx * ny, 4 << 20)
    key = (nmat, nx, ny, nz, angles, bool(scene.save_path), per_round, precision, tuple(map(tuple, (c.items() for c in candidates))))
    if key in _cache:
        return _cache[key]
    native = _native.load()
    tables = np.ascontiguousarray(scene.tables, dtype=np.float64)
    trials = []
    for c in candidates:
        config = f"precision={precision},pool={c['pool']},block={c['block']},walk={c['walk']}"
        trials.append((c, _time(native, tables, device, config, per_round, seed)))
    best, rate = max(trials, key=lambda t: t[1])
    tuned = Tuned(best["pool"], best["block"], best["walk"], rate,
                  tuple((dict(c), r) for c, r in trials))
    _cache[key] = tuned
    return tuned
