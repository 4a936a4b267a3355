"""The oracle behind the reference's Backend interface (python/monki/execution/backend.py:
10-72), so ``simulate`` can build a product from it: one round per batch, photon streams
keyed by (photon, round, seed) like the CUDA backend's. Test infrastructure only."""

from __future__ import annotations

import numpy as np


def oracle_backend(oracle, seed: int, max_steps: int = 100_000):
    from monki.execution import Backend
    from monki.execution.tallies import RawTallies

    class OracleBackend(Backend):
        def __init__(self):
            self.metadata = None
            self.provenance = {"backend": "oracle", "seed": seed}
            self.tables = None

        def prepare(self, scene):
            self.tables = np.ascontiguousarray(scene.tables)
            self.metadata = scene.metadata

        def run_batch(self, controls):
            nx, ny = int(self.tables[1]), int(self.tables[2])
            per_round = controls.photons_per_column * nx * ny
            words = [per_round, 0, controls.round_index, seed, max_steps, 0, per_round, 1]
            out, _ = oracle.run(self.tables, words)
            stokes, paths, weights = oracle.split(self.tables, out[0])
            return RawTallies(controls, stokes.copy(), None if paths is None else paths.copy(),
                              None if weights is None else weights.copy())

        def close(self):
            pass

    return OracleBackend()
