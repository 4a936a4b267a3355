"""ctypes binding of the CPU FP64 oracle (test infrastructure, not product code).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs import this module.
It builds ``monki_oracle.cpp`` on demand with ``oracle/build.py``.
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

from . import build as _build

_U32P = ctypes.POINTER(ctypes.c_uint32)
_U64P = ctypes.POINTER(ctypes.c_uint64)
_F64P = ctypes.POINTER(ctypes.c_double)
_library = None


def library() -> ctypes.CDLL:
    global _library

    if _library is None:
        path = _build.build()
        lib = ctypes.CDLL(str(path))
        lib.monki_oracle_philox.argtypes = [_U32P, _U32P, _U32P]
        lib.monki_oracle_philox.restype = None
        lib.monki_oracle_uniforms.argtypes = [ctypes.c_uint32] * 4 + [_F64P]
        lib.monki_oracle_uniforms.restype = None
        lib.monki_oracle_scatter_stokes.argtypes = [ctypes.c_double] * 5 + [_F64P, _F64P]
        lib.monki_oracle_scatter_stokes.restype = None
        lib.monki_oracle_validate.argtypes = [_F64P, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t]
        lib.monki_oracle_validate.restype = ctypes.c_int
        lib.monki_oracle_run.argtypes = [
            _F64P,
            ctypes.c_size_t,
            _U32P,
            ctypes.c_int,
            _F64P,
            _U64P,
            ctypes.c_char_p,
            ctypes.c_size_t,
        ]
        lib.monki_oracle_run.restype = ctypes.c_int
        lib.monki_oracle_run_guided.argtypes = [
            _F64P,
            ctypes.c_size_t,
            _U32P,
            _F64P,
            _F64P,
            ctypes.c_int,
            _F64P,
            _U64P,
            _F64P,
            _F64P,
            ctypes.c_uint32,
            ctypes.c_char_p,
            ctypes.c_size_t,
        ]
        lib.monki_oracle_run_guided.restype = ctypes.c_int
        _library = lib

    return _library


def philox(counter, key) -> np.ndarray:
    c = np.ascontiguousarray(counter, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    library().monki_oracle_philox(c.ctypes.data_as(_U32P), k.ctypes.data_as(_U32P), out.ctypes.data_as(_U32P))
    return out


def uniforms(photon: int, round_: int, seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.float64)
    library().monki_oracle_uniforms(photon, round_, seed, n, out.ctypes.data_as(_F64P))
    return out


def scatter_stokes(depol, uo, u1, phio, phi1, stokes) -> np.ndarray:
    s = np.ascontiguousarray(stokes, dtype=np.float64)
    out = np.zeros(3)
    library().monki_oracle_scatter_stokes(depol, uo, u1, phio, phi1, s.ctypes.data_as(_F64P), out.ctypes.data_as(_F64P))
    return out


def validate(tables) -> str | None:
    t = np.ascontiguousarray(tables, dtype=np.float64)
    err = ctypes.create_string_buffer(1024)
    status = library().monki_oracle_validate(t.ctypes.data_as(_F64P), t.size, err, len(err))
    return err.value.decode() if status else None


def tally_count(tables, orders: bool = False) -> int:
    nx, ny, nz, nmat, angles = (int(v) for v in tables[1:6])
    paths = bool(tables[10])
    count = nmat * nx * ny * angles + (nx * ny * (nz + 1) * angles if paths else 0)
    if orders:
        count += nmat * nx * ny * angles + 2 * nmat * nx * ny * nz * angles
    return count


def run(tables, controls, threads: int | None = None, guide=None, scale=None, importance: bool = False,
        pixel_weights=None, orders: bool = False):
    """Run one round group; returns (tallies[rounds, tally_count], counters dict[, importance]).

    ``controls`` are the eight words of the CUDA run call. ``guide`` = (epsilon, roulette
    [, DDIS weight cap[, splitting factor]]) selects guided transport (detector-directed
    sampling at particle scatters, Russian roulette and splitting); None is the analog
    method. ``scale`` (nx, ny, nz),
    Fortran order, multiplies the roulette weight per cell. With ``importance`` the third
    result is the importance tally, shape (2, nx, ny, nz): summed future contribution per
    unit weight and event count per cell, each contribution weighted by ``pixel_weights``
    (nx, ny, angles) of its output pixel when given. ``orders`` appends the scattering-order
    diagnostics to each round (see ``split_orders``). A failure flag raises.
    """

    t = np.ascontiguousarray(tables, dtype=np.float64)
    ctl = np.ascontiguousarray(controls, dtype=np.uint32)
    nx, ny, nz = (int(v) for v in t[1:4])
    rounds = int(ctl[7])
    out = np.zeros((rounds, tally_count(t, orders)), dtype=np.float64)
    counters = np.zeros(5, dtype=np.uint64)
    err = ctypes.create_string_buffer(4096)
    threads = threads or os.cpu_count() or 1
    g = np.zeros(4)
    g[: len(guide or ())] = guide or ()
    scale_arr = None if scale is None else np.ascontiguousarray(np.asarray(scale, dtype=np.float64).ravel(order="F"))
    if scale_arr is not None and scale_arr.size != nx * ny * nz:
        raise ValueError("scale must have nx * ny * nz cells")
    imp = np.zeros(2 * nx * ny * nz) if importance else None
    angles = int(t[5])
    weights_arr = None
    if pixel_weights is not None:
        weights_arr = np.ascontiguousarray(np.asarray(pixel_weights, dtype=np.float64).ravel(order="F"))
        if weights_arr.size != nx * ny * angles:
            raise ValueError("pixel_weights must have nx * ny * angles values")
    status = library().monki_oracle_run_guided(
        t.ctypes.data_as(_F64P),
        t.size,
        ctl.ctypes.data_as(_U32P),
        g.ctypes.data_as(_F64P),
        None if scale_arr is None else scale_arr.ctypes.data_as(_F64P),
        threads,
        out.ctypes.data_as(_F64P),
        counters.ctypes.data_as(_U64P),
        None if imp is None else imp.ctypes.data_as(_F64P),
        None if weights_arr is None else weights_arr.ctypes.data_as(_F64P),
        1 if orders else 0,
        err,
        len(err),
    )

    if status:
        raise RuntimeError(err.value.decode() or f"oracle failed with flag {status}")

    names = ("scatters", "photons", "free_path_visits", "detector_visits", "tally_updates")
    stats = {name: int(value) for name, value in zip(names, counters, strict=True)}
    if importance:
        cells = nx * ny * nz
        return out, stats, np.stack([imp[:cells].reshape((nx, ny, nz), order="F"), imp[cells:].reshape((nx, ny, nz), order="F")])
    return out, stats


def split_orders(tables, values):
    """The scattering-order block of one round: (single-scattering Stokes (nmat, nx, ny,
    angles), contributions by event location and of single scattering (nmat, nx, ny, nz,
    angles each, layer 0 = the surface))."""

    nx, ny, nz, nmat, angles = (int(v) for v in tables[1:6])
    at = tally_count(tables)
    s = nmat * nx * ny * angles
    loc = nmat * nx * ny * nz * angles
    single = values[at : at + s].reshape((nmat, nx, ny, angles), order="F")
    located = values[at + s : at + s + loc].reshape((nmat, nx, ny, nz, angles), order="F")
    located_single = values[at + s + loc : at + s + 2 * loc].reshape((nmat, nx, ny, nz, angles), order="F")
    return single, located, located_single


def split(tables, values):
    """Split one round's flat tallies into (stokes, paths, weights) Fortran-order arrays."""

    nx, ny, nz, nmat, angles = (int(v) for v in tables[1:6])
    stokes_count = nmat * nx * ny * angles
    stokes = values[:stokes_count].reshape((nmat, nx, ny, angles), order="F")

    if not bool(tables[10]):
        return stokes, None, None

    path_count = nx * ny * nz * angles
    paths = values[stokes_count : stokes_count + path_count].reshape((nx, ny, nz, angles), order="F")
    weights = values[stokes_count + path_count :].reshape((nx, ny, angles), order="F")
    return stokes, paths, weights


ROOT = Path(__file__).resolve().parent
