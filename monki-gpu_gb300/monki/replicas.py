"""Replicas: statistical rounds split across processes (one per GPU), one FP64 sum.

A run shards by statistical round. Each round has its own random streams (Philox counters
keyed by round and photon, kernels/metal/transport.metal:352-357) and is a complete,
independent sample (python/monki/simulation.py:30-33), so ranks run disjoint round
indices through their own backends and the only exchange is one all-reduce of the FP64
round moments: the Stokes sums, the sums of squares of the per-round radiance, and the
path and weight sums. The result equals one process running the same rounds (the sums
differ only in FP64 summation order); radiance and standard error follow the reference
driver (simulation.py:73-156, main.f90:1405-1451).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .execution.tallies import RawTallies

SENTINEL_ROUNDS = 30  # the standard error is 999 until more rounds than this have run


def rank_rounds(total_rounds: int, rank: int, world: int) -> list[int]:
    """Round indices (from 1) that rank `rank` of `world` runs: every world-th round."""

    if not (0 <= rank < world) or total_rounds < 0:
        raise ValueError("rank must be in [0, world) and total_rounds non-negative")
    return list(range(rank + 1, total_rounds + 1, world))


@dataclass
class RoundMoments:
    rounds: int
    photons_per_column: int
    stokes: np.ndarray          # sum over rounds of the Stokes tallies (nmat, nx, ny, angles)
    squares: np.ndarray         # sum over rounds of (Stokes / photons per column)^2
    paths: np.ndarray | None    # sum of the layer-path tallies (nx, ny, nz, angles)
    weights: np.ndarray | None  # sum of the detected weights (nx, ny, angles)

    @classmethod
    def of(cls, batches: list[RawTallies], photons_per_column: int) -> RoundMoments:
        if not batches:
            raise ValueError("no rounds")
        stokes = np.zeros_like(batches[0].stokes, dtype=np.float64)
        squares = np.zeros_like(stokes)
        paths = None if batches[0].weighted_paths is None else np.zeros_like(batches[0].weighted_paths, dtype=np.float64)
        weights = None if batches[0].weights is None else np.zeros_like(batches[0].weights, dtype=np.float64)
        for batch in batches:
            if batch.controls.photons_per_column != photons_per_column:
                raise ValueError("every round must use the same photons per column")
            stokes += batch.stokes
            squares += (batch.stokes / photons_per_column) ** 2
            if paths is not None:
                paths += batch.weighted_paths
                weights += batch.weights
        return cls(len(batches), photons_per_column, stokes, squares, paths, weights)

    def estimate(self):
        """(radiance, standard error) of the rounds, Fortran order (nmat, nx, ny, angles)."""

        n = self.rounds
        x = self.stokes / self.photons_per_column
        radiance = x / n
        if n <= SENTINEL_ROUNDS:
            return radiance, np.full_like(radiance, 999.0)
        error = np.sqrt(np.maximum(self.squares - x * x / n, 0.0) / (n - 1)) / np.sqrt(n)
        return radiance, error


def all_reduce(moments: RoundMoments, group=None) -> RoundMoments:
    """Sum every rank's moments (torch.distributed, FP64, one collective): on CPU tensors
    for gloo, on the current CUDA device for nccl."""

    import torch
    import torch.distributed as dist

    parts = [np.array([moments.rounds], dtype=np.float64), moments.stokes.ravel(), moments.squares.ravel()]
    if moments.paths is not None:
        parts += [moments.paths.ravel(), moments.weights.ravel()]
    flat = torch.from_numpy(np.concatenate(parts))
    if dist.get_backend(group) == "nccl":
        flat = flat.cuda()
    dist.all_reduce(flat, op=dist.ReduceOp.SUM, group=group)
    values = flat.cpu().numpy()
    at = 1

    def take(like):
        nonlocal at
        out = values[at : at + like.size].reshape(like.shape).copy()
        at += like.size
        return out

    stokes, squares = take(moments.stokes), take(moments.squares)
    paths = weights = None
    if moments.paths is not None:
        paths, weights = take(moments.paths), take(moments.weights)
    return RoundMoments(int(round(values[0])), moments.photons_per_column, stokes, squares, paths, weights)
