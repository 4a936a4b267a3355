"""The reference's archived Fortran runs as statistical goldens (test infrastructure).

``tests/golden/archived_<name>.npz`` holds, for each of the three runs archived with the
reference (fortran/monki/upstream/OUTPUT/testrun/*.nc): its radiance and standard error
(ang, y, x, nmat, band order, as the file stores them), its settings, the Fortran
preparer's optical depths, and the table stream monki.preparation builds for the same run
with the first group of view zeniths. The runs have up to 90 views and a device scene holds
16, so each group of views runs as its own scene: a view's peel-off never depends on the
other views, so its estimate is the same whichever views share the run.

The Fortran's estimate of a run (main.f90:1405-1451): per round X = Stokes / photons per
column; radiance = mean of X over the rounds; standard error =
sqrt((sum X^2 - (sum X)^2 / n) / (n - 1)) / sqrt(n).
"""

from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
NAMES = ("cloudfree", "1layercloud", "2boxclouds")


def load(name: str) -> dict:
    with np.load(GOLDEN / f"archived_{name}.npz") as data:
        return {key: data[key] for key in data.files}


def with_views(tables: np.ndarray, zeniths) -> np.ndarray:
    """The table stream with its view zeniths replaced (same count; version >= 2 stream:
    header, geometry, layer thicknesses, then the view zeniths)."""

    tables = np.array(tables, dtype=np.float64, copy=True)
    version, nz, angles = int(tables[0]), int(tables[3]), int(tables[5])
    zeniths = np.asarray(zeniths, dtype=np.float64)
    if version < 2 or zeniths.size > angles:
        raise ValueError("view group larger than the prepared scene")
    if zeniths.size < angles:
        # Fewer views than the prepared scene: shrink the view blocks of the stream.
        start = 18 + nz
        azimuth = tables[start + angles]
        tables = np.concatenate([tables[:start], zeniths, np.full(zeniths.size, azimuth), tables[start + 2 * angles:]])
        tables[5] = zeniths.size
        return tables
    tables[18 + nz : 18 + nz + angles] = zeniths
    return tables


def view_groups(fixture: dict):
    return [(int(lo), int(hi)) for lo, hi in fixture["view_groups"]]


def round_statistics(stokes_rounds: np.ndarray, photons_per_column: int):
    """Radiance and its standard error in the archived layout from per-round Stokes
    tallies of shape (rounds, nmat, nx, ny, angles)."""

    x = np.asarray(stokes_rounds, dtype=np.float64) / photons_per_column
    n = x.shape[0]
    total, squares = x.sum(0), (x * x).sum(0)
    radiance = total / n
    error = np.sqrt(np.maximum(squares - total * total / n, 0.0) / (n - 1)) / np.sqrt(n)
    return radiance.transpose(3, 2, 1, 0), error.transpose(3, 2, 1, 0)


def z_scores(radiance, error, fixture, views=slice(None)):
    """(ours - archived) / combined standard error, over entries with a nonzero error."""

    archived = fixture["radiance"][views, ..., 0]
    archived_error = fixture["std_radiance"][views, ..., 0]
    combined = np.hypot(error, archived_error)
    mask = combined > 0
    return (radiance - archived)[mask] / combined[mask]


def bonferroni_bound(entries: int, family_error: float = 1e-6) -> float:
    """|z| that a family of `entries` two-sided tests exceeds with probability family_error."""

    from scipy.stats import norm

    return float(norm.isf(family_error / (2 * entries)))
