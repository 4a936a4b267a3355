"""The FP32 bias of a result, stated against the FP64 transport build.

The product transport runs in FP32 (FP64 tallies, flush and statistics); the same
kernels compiled for FP64 (``CUDA(precision="fp64")``) are kept as the check build. For
a scene, both run the same number of rounds with independent streams, and the bias of
each Stokes component (and of the layer AMF with path diagnostics) is the mean relative
difference FP32 - FP64 over pixels and views, with its standard error from the round-to-
round spread, plus the share of entries whose difference exceeds three combined
standard errors (expected about 0.3 % without bias).
"""

from __future__ import annotations

import numpy as np


def _rounds(scene, precision, rounds, photons_per_column, seed, device):
    from .execution import CUDA, BatchControls

    with CUDA(device=device, precision=precision, seed=seed) as backend:
        backend.prepare(scene)
        batches = backend.run_batches([BatchControls(i, photons_per_column) for i in range(1, rounds + 1)])
    stokes = np.stack([b.stokes for b in batches]) / photons_per_column
    amf = None
    if batches[0].weighted_paths is not None:
        amf = np.stack([b.weighted_paths[:, :, :-1, :] / b.weights[:, :, None, :] for b in batches])
    return stokes, amf


def _compare(a, b):
    n = a.shape[0]
    ma, mb = a.mean(0), b.mean(0)
    se = np.hypot(a.std(0, ddof=1), b.std(0, ddof=1)) / np.sqrt(n)
    scale = np.abs(mb)
    mask = (scale > 1e-12) & (se > 0)
    relative = (ma - mb)[mask] / scale[mask]
    relative_se = se[mask] / scale[mask]
    weights = 1.0 / relative_se**2
    mean = float(np.sum(weights * relative) / np.sum(weights))
    return {
        "relative_bias": mean,
        "relative_bias_se": float(1.0 / np.sqrt(np.sum(weights))),
        "share_beyond_3_se": float(np.mean(np.abs((ma - mb)[mask] / se[mask]) > 3)),
        "entries": int(mask.sum()),
    }


def fp32_bias(scene, *, rounds: int = 8, photons_per_column: int = 2000, device: int = 0, seed: int = 101) -> dict:
    """FP32 - FP64 relative difference per Stokes component (and for the layer AMF)."""

    s32, a32 = _rounds(scene, "fp32", rounds, photons_per_column, seed, device)
    s64, a64 = _rounds(scene, "fp64", rounds, photons_per_column, seed + 1, device)
    names = ("I", "Q", "U")[: s32.shape[1]]
    out = {name: _compare(s32[:, m], s64[:, m]) for m, name in enumerate(names)}
    if a32 is not None:
        out["AMF"] = _compare(a32, a64)
    out["rounds"] = rounds
    out["photons_per_column"] = photons_per_column
    return out
