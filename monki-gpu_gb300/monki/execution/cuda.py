"""GB300 transport backend: every photon history runs in the sm_103a kernels.

``CUDA`` mirrors the reference's ``Metal`` backend (python/monki/execution/metal.py:23-349):
settings validated eagerly, ``prepare`` uploads resident tables once, equal-size rounds
are grouped into one launch with independent random streams and tallies, requests are
validated before any device work, and any native failure closes the session. The device
flushes FP32 tally banks into FP64 per-round sums, so the host only copies results out.
There is no CPU path: a missing library, a missing GPU or a failed launch raises.
"""

from __future__ import annotations

import ctypes
import hashlib
import os
import platform

import numpy as np

from ..guided import Guided
from ..input import ReferenceCase
from ..scenes import TransportScene
from . import native as _native

_DIGESTS: dict = {}


def _library_digest(path) -> str:
    """SHA-256 of the native library file, computed once per file version in a process (the
    receipts carry it; hashing the library on every prepare cost a few milliseconds)."""

    stat = os.stat(path)
    key = (os.fspath(path), stat.st_size, stat.st_mtime_ns)
    if key not in _DIGESTS:
        with open(path, "rb") as f:
            _DIGESTS[key] = hashlib.sha256(f.read()).hexdigest()
    return _DIGESTS[key]
from .backend import Backend
from .tallies import BatchControls, RawTallies

_PRECISIONS = ("fp32", "fp64")


class CUDA(Backend):
    """Resident GB300 transport session; one caller per instance.

    ``precision="fp32"`` is the production transport. ``"fp64"`` runs the same kernels in
    double precision: it is the on-device check build against which the FP32 bias of
    each result is stated.

    ``guided`` (a ``Guided``) turns on importance-guided transport: detector-directed
    sampling at particle scatters and Russian roulette, both with exact weight correction;
    ``set_roulette_scale`` gives the roulette weight a per-cell scale. ``importance=True``
    makes the session tally per-cell detector importance (``importance()``), the training
    data of the learned importance model.
    """

    def __init__(
        self,
        device: int = 0,
        *,
        save_path: bool | None = None,
        profile: bool = False,
        seed: int = 23274,
        photons_per_dispatch: int = 1 << 30,
        tally_shards: int = 8,
        max_steps: int = 100_000,
        precision: str = "fp32",
        block: int = 256,
        engine: str = "wavefront",
        pool: int = 1 << 22,
        walk: int = 3,
        guided: Guided | None = None,
        importance: bool = False,
        roulette_scale=None,
        device_statistics: bool = True,
        orders: bool = False,
        rectangles: bool = True,
        tail: int = 1 << 16,
        lookahead: bool = True,
        monki_home=None,
        library=None,
    ):
        for name, value, minimum, maximum in (
            ("device", device, 0, 2**32 - 1),
            ("seed", seed, 0, 2**32 - 1),
            ("tally_shards", tally_shards, 1, 64),
            ("photons_per_dispatch", photons_per_dispatch, 1, 2**31 - 1),
            ("max_steps", max_steps, 1, 10_000_000),
            ("block", block, 32, 256),
            ("tail", tail, 0, 1 << 26),
        ):
            if type(value) is not int or not minimum <= value <= maximum:
                raise ValueError(f"{name} must be an integer in [{minimum}, {maximum}]")

        if save_path is not None and type(save_path) is not bool:
            raise ValueError("save_path must be a bool or None")

        if type(profile) is not bool:
            raise ValueError("profile must be a bool")

        if precision not in _PRECISIONS:
            raise ValueError("precision must be 'fp32' or 'fp64'")

        if block % 32:
            raise ValueError("block must be a multiple of 32")

        if engine not in ("wavefront", "megakernel"):
            raise ValueError("engine must be 'wavefront' or 'megakernel'")

        if type(pool) is not int or not 1024 <= pool <= 1 << 26:
            raise ValueError("pool must be an integer in [1024, 2**26]")

        if type(walk) is not int or not 1 <= walk <= 1 << 20:
            raise ValueError("walk must be an integer in [1, 2**20]")

        if guided is not None and not isinstance(guided, Guided):
            raise ValueError("guided must be a monki.Guided or None")

        if type(importance) is not bool:
            raise ValueError("importance must be a bool")

        if (guided is not None or importance) and engine != "wavefront":
            raise ValueError("guided transport and importance tallies need engine='wavefront'")

        if type(orders) is not bool:
            raise ValueError("orders must be a bool")

        if orders and engine != "wavefront":
            raise ValueError("scattering-order diagnostics need engine='wavefront'")

        if type(rectangles) is not bool:
            raise ValueError("rectangles must be a bool")

        if type(lookahead) is not bool:
            raise ValueError("lookahead must be a bool")

        self.device = device
        self.save_path = save_path
        self.profile = profile
        self.seed = seed
        self.photons_per_dispatch = photons_per_dispatch
        self.tally_shards = tally_shards
        self.max_steps = max_steps
        self.precision = precision
        self.block = block
        self.engine = engine
        self.pool = pool
        self.walk = walk
        self.guided = guided
        self.importance_tally = importance
        # simulate() folds rounds into FP64 statistics on the device when available.
        self.device_statistics = bool(device_statistics)
        # Scattering-order diagnostics (single / multiple scattering, contribution by event
        # location), the reference's save_scats outputs.
        self.orders = orders
        # The free-path walk crosses each rectangle of equal-extinction cells of a horizontally
        # varying layer in one step (the same path in exact arithmetic as the face-by-face
        # walk); False keeps the face-by-face walk.
        self.rectangles = rectangles
        # A round group's last photons (at most this many, every photon claimed) run to their
        # ends in one tail launch; 0 keeps the wavefront launches to the end.
        self.tail = tail
        # simulate() with a stopping rule runs, after the first check, the rounds the last
        # check says are still needed in one held dispatch, folded and checked one by one.
        self.lookahead = lookahead
        self.monki_home = monki_home
        # Per-cell roulette scale (nx, ny, nz) applied at every prepare; set_roulette_scale
        # changes it for the prepared session only.
        self.roulette_scale = None if roulette_scale is None else np.asarray(roulette_scale, dtype=np.float64)
        self.library = library or _native.LIBRARY
        self.metadata = None
        self.provenance: dict = {}
        self._native = None
        self._handle = None
        self._shape = (0, 0, 0, 0, 0)
        self._paths = False
        self._configuration = None
        self._round = 0
        self._tally_count = 0
        self._round_capacity = 1

    # ------------------------------------------------------------------ lifecycle
    def prepare(self, scene: object) -> None:
        """Validate the prepared tables, upload them once and size the round banks."""

        self.close()

        if isinstance(scene, ReferenceCase):
            # A reference fixture: prepare its tables on the host (monki.preparation), from
            # the MONKI home directory that holds INPUT/ and DATA/.
            home = self.monki_home or os.environ.get("MONKI_HOME")

            if not home:
                raise ValueError("preparing a ReferenceCase needs monki_home= or MONKI_HOME (the directory with INPUT/ and DATA/)")

            from ..preparation import prepare_reference_case

            scene = prepare_reference_case(scene, home)

        if not isinstance(scene, TransportScene):
            raise TypeError("CUDA.prepare expects a TransportScene or a ReferenceCase")

        tables = np.array(scene.tables, dtype=np.float64, copy=True)

        if tables.ndim != 1 or tables.size < 18 or not np.all(np.isfinite(tables)):
            raise ValueError("Invalid/nonfinite prepared transport export")

        if bool(scene.backward) != bool(tables[11]):
            raise ValueError("scene.backward disagrees with the backward flag of its table stream")

        if scene.backward and (self.guided is not None or self.importance_tally):
            raise ValueError("guided transport and importance tallies need forward transport")

        if self.save_path is not None:
            tables[10] = float(self.save_path)

        nx, ny, nz, nmat, angles = (int(v) for v in tables[1:6])
        paths = bool(tables[10])
        tally_count = nmat * nx * ny * angles + (nx * ny * (nz + 1) * angles if paths else 0)
        if self.orders:
            tally_count += nmat * nx * ny * angles + 2 * nmat * nx * ny * nz * angles
        per_round = scene.photons_per_column * nx * ny
        # Device tally records per round and shard: {I, Q, U, weight} per pixel, plus
        # {layer, view, first, -} per (pixel, layer + 1) with path diagnostics.
        pixels = nx * ny * angles
        device_count = 4 * pixels + (4 * pixels * (nz + 1) if paths else 0)
        if self.orders:
            device_count += 4 * (pixels + 2 * nx * ny * nz * angles)
        bytes_per_round = device_count * self.tally_shards * (4 if self.precision == "fp32" else 8)
        capacity = max(
            1,
            min(
                64,
                self.photons_per_dispatch // max(per_round, 1),
                (1 << 30) // max(bytes_per_round, 1),
            ),
        )
        native = _native.load(self.library)
        error = ctypes.create_string_buffer(8192)
        config = (
            f"precision={self.precision},shards={self.tally_shards},block={self.block},"
            f"engine={self.engine},pool={self.pool},walk={self.walk},tail={self.tail}"
            + (self.guided.config() if self.guided is not None else "")
            + (",importance=1" if self.importance_tally else "")
            + (",orders=1" if self.orders else "")
            + ("" if self.rectangles else ",rectangles=0")
        ).encode()
        handle = native.monki_cuda_create(
            self.device,
            tables.ctypes.data_as(_native.F64P),
            tables.size,
            capacity,
            config,
            error,
            len(error),
        )

        if not handle:
            raise RuntimeError(error.value.decode() or "CUDA session creation failed")

        self._native = native
        self._handle = handle
        self._shape = (nmat, nx, ny, nz, angles)
        self._paths = paths
        self._tally_count = int(native.monki_cuda_tally_count(handle))
        self._round_capacity = capacity
        self._round = 0
        self._configuration = self._settings()
        self.metadata = scene.metadata

        if self._tally_count != tally_count:
            self.close()
            raise RuntimeError("CUDA tally layout disagrees with the prepared tables")

        self.provenance = {
            "backend": "CUDA",
            "device": native.monki_cuda_device_name(handle).decode(),
            "scene": scene.name,
            "rng": "Philox4x32-10; seed/round/photon/draw-block",
            "seed": self.seed,
            "transport_precision": "float32" if self.precision == "fp32" else "float64",
            "tally_precision": "float32 banks, float64 per-round flush"
            if self.precision == "fp32"
            else "float64",
            "round_precision": "float64",
            "photons_per_dispatch": self.photons_per_dispatch,
            "tally_shards": self.tally_shards,
            "round_capacity": capacity,
            "max_steps": self.max_steps,
            "block": self.block,
            "engine": self.engine,
            "pool": self.pool,
            "walk": self.walk,
            "guided": None if self.guided is None else self.guided.describe(),
            "library_sha256": _library_digest(self.library),
            "tables_sha256": hashlib.sha256(tables.tobytes()).hexdigest(),
            "machine": platform.machine(),
            "python_version": platform.python_version(),
            "gpu_dispatches": 0,
            "scatters": 0,
            "photons": 0,
            "kernel_launches": 0,
        }

        if self.roulette_scale is not None:
            try:
                self.set_roulette_scale(self.roulette_scale)
            except Exception:
                self.close()
                raise

    def set_roulette_scale(self, scale) -> None:
        """Scale the guided roulette weight per cell: ``scale`` has shape (nx, ny, nz)
        (the vacuum layer included); None removes the map. Applies to later rounds."""

        if self._handle is None:
            raise RuntimeError("CUDA backend has no prepared scene")

        error = ctypes.create_string_buffer(8192)

        if scale is None:
            status = self._native.monki_cuda_set_roulette_scale(self._handle, None, 0, error, len(error))
        else:
            _, nx, ny, nz, _ = self._shape
            values = np.asarray(scale, dtype=np.float64)

            if values.shape != (nx, ny, nz):
                raise ValueError(f"roulette scale must have shape {(nx, ny, nz)}")

            flat = np.ascontiguousarray(values.ravel(order="F"))
            status = self._native.monki_cuda_set_roulette_scale(
                self._handle, flat.ctypes.data_as(_native.F64P), flat.size, error, len(error)
            )

        if status:
            raise RuntimeError(error.value.decode() or "setting the roulette scale failed")

        self.provenance["roulette_scale"] = None if scale is None else "per-cell map"

    def set_importance_weights(self, weights) -> None:
        """Weight the importance tally's contributions per output pixel: ``weights`` has
        shape (nx, ny, angles); None restores equal weights."""

        if self._handle is None:
            raise RuntimeError("CUDA backend has no prepared scene")

        error = ctypes.create_string_buffer(8192)

        if weights is None:
            status = self._native.monki_cuda_set_importance_weights(self._handle, None, 0, error, len(error))
        else:
            _, nx, ny, _, angles = self._shape
            values = np.asarray(weights, dtype=np.float64)

            if values.shape != (nx, ny, angles):
                raise ValueError(f"importance weights must have shape {(nx, ny, angles)}")

            flat = np.ascontiguousarray(values.ravel(order="F"))
            status = self._native.monki_cuda_set_importance_weights(
                self._handle, flat.ctypes.data_as(_native.F64P), flat.size, error, len(error)
            )

        if status:
            raise RuntimeError(error.value.decode() or "setting the importance weights failed")

    def importance(self, reset: bool = True) -> np.ndarray:
        """The importance tally of the rounds run so far: shape (2, nx, ny, nz), the summed
        future Stokes-I contribution per unit weight and the event count of each cell."""

        if self._handle is None:
            raise RuntimeError("CUDA backend has no prepared scene")

        _, nx, ny, nz, _ = self._shape
        cells = nx * ny * nz
        out = np.zeros(2 * cells)
        error = ctypes.create_string_buffer(8192)

        if self._native.monki_cuda_importance(
            self._handle, out.ctypes.data_as(_native.F64P), out.size, int(reset), error, len(error)
        ):
            raise RuntimeError(error.value.decode() or "reading the importance tally failed")

        return np.stack([out[:cells].reshape((nx, ny, nz), order="F"), out[cells:].reshape((nx, ny, nz), order="F")])

    def run_batch(self, controls: object) -> RawTallies:
        """Execute exactly one complete statistical round."""

        return self._run_group([controls])[0]

    def run_batches(self, controls: list) -> list:
        """Group consecutive equal-size rounds into shared launches, preserving order."""

        self._validate_requests(controls)
        results = []
        first = 0
        _, nx, ny, _, _ = self._shape

        while first < len(controls):
            photons = controls[first].photons_per_column * nx * ny
            capacity = max(1, min(self._round_capacity, self.photons_per_dispatch // photons))
            last = first + 1

            while last < min(len(controls), first + capacity):
                if controls[last].photons_per_column != controls[first].photons_per_column:
                    break

                last += 1

            results.extend(self._run_group(controls[first:last]))
            first = last

        return results

    # ------------------------------------------------------------------ device statistics
    def device_statistics_available(self, photons_per_column: int) -> bool:
        """True when whole rounds of this size fit one dispatch, so the device can fold
        each round into its FP64 statistics (``accumulate``)."""

        _, nx, ny, _, _ = self._shape
        return (self.device_statistics and not self.orders
                and photons_per_column * nx * ny <= self.photons_per_dispatch)

    def accumulate(self, controls: list) -> np.ndarray:
        """Run rounds and fold their tallies into the device's FP64 round statistics
        without copying them to the host. Returns, per round, the spatial sum of the
        round's normalized Stokes tallies (rounds x nmat)."""

        self._validate_requests(controls)
        nmat, nx, ny, _, _ = self._shape
        history = []
        first = 0

        while first < len(controls):
            ppc = controls[first].photons_per_column
            per_round = ppc * nx * ny

            if per_round > self.photons_per_dispatch:
                raise ValueError("device statistics need whole rounds in one dispatch")

            capacity = max(1, min(self._round_capacity, self.photons_per_dispatch // per_round))
            last = first + 1

            while last < min(len(controls), first + capacity) and controls[last].photons_per_column == ppc:
                last += 1

            group = controls[first:last]
            rows = np.zeros((len(group), nmat), dtype=np.float64)
            error = ctypes.create_string_buffer(8192)
            command = (ctypes.c_uint32 * 8)(
                per_round * len(group), 0, group[0].round_index, self.seed, self.max_steps, int(self.profile),
                per_round, len(group),
            )

            try:
                status = self._native.monki_cuda_run_accumulate(
                    self._handle, command, float(ppc), rows.ctypes.data_as(_native.F64P), error, len(error)
                )

                if status or not np.all(np.isfinite(rows)):
                    raise RuntimeError(error.value.decode() or "Nonfinite CUDA tallies")
            except BaseException:
                self.close()
                raise

            self.provenance["gpu_dispatches"] += 1
            history.append(rows)
            self._round = group[-1].round_index
            first = last

        counters = (ctypes.c_uint64 * 6)()
        self._native.monki_cuda_counters(self._handle, counters)
        self.provenance["scatters"] = int(counters[0])
        self.provenance["photons"] = int(counters[4])
        self.provenance["kernel_launches"] = int(counters[5])

        if self.profile:
            self.provenance["gpu_seconds"] = self._native.monki_cuda_gpu_seconds(self._handle)

        return np.concatenate(history) if history else np.zeros((0, nmat))

    def held_capacity(self, photons_per_column: int) -> int:
        """How many rounds of this size one held group (``run_held``) can run."""

        _, nx, ny, _, _ = self._shape
        return max(1, min(self._round_capacity, self.photons_per_dispatch // max(1, photons_per_column * nx * ny)))

    def run_held(self, controls: list) -> None:
        """Run consecutive rounds (one dispatch) ahead of their stopping checks: their tallies
        stay on the device, unfolded, until ``fold_next`` folds them one by one in round order;
        the ones never folded are discarded by the next run. The same rounds, folds and
        checks as dispatching the rounds one at a time, with the straggler tail of a dispatch
        paid once per group."""

        self._validate_requests(controls)
        _, nx, ny, _, _ = self._shape
        ppc = controls[0].photons_per_column
        if any(c.photons_per_column != ppc for c in controls) or any(
            b.round_index != a.round_index + 1 for a, b in zip(controls, controls[1:])
        ):
            raise ValueError("a held group is consecutive rounds of one size")
        if len(controls) > self.held_capacity(ppc):
            raise ValueError("held group larger than one dispatch")
        per_round = ppc * nx * ny
        command = (ctypes.c_uint32 * 8)(
            per_round * len(controls), 0, controls[0].round_index, self.seed, self.max_steps, int(self.profile),
            per_round, len(controls),
        )
        error = ctypes.create_string_buffer(8192)
        try:
            if self._native.monki_cuda_run_held(self._handle, command, error, len(error)):
                raise RuntimeError(error.value.decode() or "CUDA transport failed")
        except BaseException:
            self.close()
            raise
        self.provenance["gpu_dispatches"] += 1
        self._held = [c.photons_per_column for c in controls]
        self._round = controls[-1].round_index
        counters = (ctypes.c_uint64 * 6)()
        self._native.monki_cuda_counters(self._handle, counters)
        self.provenance["scatters"] = int(counters[0])
        self.provenance["photons"] = int(counters[4])
        self.provenance["kernel_launches"] = int(counters[5])

    def fold_next(self) -> np.ndarray:
        """Fold the next held round into the device statistics; returns its nmat spatial
        sums of the normalized Stokes tallies."""

        if not getattr(self, "_held", None):
            raise RuntimeError("no held round left to fold")
        nmat = self._shape[0]
        row = np.zeros(nmat, dtype=np.float64)
        error = ctypes.create_string_buffer(8192)
        ppc = self._held.pop(0)
        if self._native.monki_cuda_fold_next(self._handle, float(ppc), row.ctypes.data_as(_native.F64P), error,
                                             len(error)):
            raise RuntimeError(error.value.decode() or "folding the held round failed")
        if not np.all(np.isfinite(row)):
            raise RuntimeError("Nonfinite CUDA tallies")
        return row

    def statistics(self) -> dict:
        """The device's FP64 round statistics: ``rounds`` and, in RawTallies shapes, the
        Stokes ``total``, ``sum`` and ``squares`` of the normalized tallies, and with path
        diagnostics the path and weight sums and their Welford moments (``path_mean``,
        ``path_m2``, ``covariance``, ``weight_mean``, ``weight_m2``)."""

        if self._handle is None:
            raise RuntimeError("CUDA backend has no prepared scene")

        nmat, nx, ny, nz, angles = self._shape
        count = int(self._native.monki_cuda_statistics_count(self._handle))
        values = np.zeros(count)
        rounds = ctypes.c_uint64(0)
        error = ctypes.create_string_buffer(8192)

        if self._native.monki_cuda_statistics(self._handle, values.ctypes.data_as(_native.F64P), count,
                                              ctypes.byref(rounds), error, len(error)):
            raise RuntimeError(error.value.decode() or "reading the statistics failed")

        s, p, w = nmat * nx * ny * angles, (nx * ny * nz * angles if self._paths else 0), (nx * ny * angles if self._paths else 0)
        at = 0

        def take(n, shape):
            nonlocal at
            out = values[at : at + n].reshape(shape, order="F").copy()
            at += n
            return out

        out = {"rounds": int(rounds.value)}
        for name in ("total", "sum", "squares"):
            out[name] = take(s, (nmat, nx, ny, angles))
        if self._paths:
            for name in ("paths", "path_mean", "path_m2", "covariance"):
                out[name] = take(p, (nx, ny, nz, angles))
            for name in ("weights", "weight_mean", "weight_m2"):
                out[name] = take(w, (nx, ny, angles))
        return out

    def reset_statistics(self) -> None:
        if self._handle is not None:
            self._native.monki_cuda_reset_statistics(self._handle)

    def close(self) -> None:
        """Release device memory; returned arrays stay valid."""

        if self._handle is not None and self._native is not None:
            self._native.monki_cuda_close(self._handle)

        self._handle = None
        self._native = None
        self.metadata = None
        self._configuration = None

    # ------------------------------------------------------------------ internals
    def _settings(self) -> tuple:
        return (
            self.device,
            self.save_path,
            self.seed,
            self.photons_per_dispatch,
            self.max_steps,
            self.profile,
            self.tally_shards,
            self.precision,
            self.block,
            self.engine,
            self.pool,
            self.walk,
            self.orders,
            self.rectangles,
            self.tail,
            self.guided,
            self.importance_tally,
        )

    def _validate_requests(self, controls: list) -> None:
        if self._handle is None or self._native is None:
            raise RuntimeError("CUDA must be prepared before running a batch")

        if self._settings() != self._configuration:
            raise ValueError("CUDA settings changed; reprepare before running another batch")

        _, nx, ny, _, _ = self._shape

        for offset, request in enumerate(controls, start=1):
            if not isinstance(request, BatchControls):
                raise TypeError("run_batch expects BatchControls")

            if request.round_index != self._round + offset:
                raise ValueError("round_index must be sequential, starting at one")

            if request.photons_per_column * nx * ny >= 2**32:
                raise ValueError("CUDA photon identity exceeds its 32-bit round range")

    def _run_group(self, controls: list) -> list[RawTallies]:
        self._validate_requests(controls)
        assert self._native is not None
        nmat, nx, ny, nz, angles = self._shape
        per_round = controls[0].photons_per_column * nx * ny
        photon_count = per_round * len(controls)
        total = np.zeros((len(controls), self._tally_count), dtype=np.float64)
        scratch = np.empty_like(total)
        error = ctypes.create_string_buffer(8192)

        try:
            for first in range(0, photon_count, self.photons_per_dispatch):
                count = min(self.photons_per_dispatch, photon_count - first)
                command = (ctypes.c_uint32 * 8)(
                    count,
                    first,
                    controls[0].round_index,
                    self.seed,
                    self.max_steps,
                    int(self.profile),
                    per_round,
                    len(controls),
                )
                status = self._native.monki_cuda_run(
                    self._handle, command, scratch.ctypes.data_as(_native.F64P), error, len(error)
                )

                if status or not np.all(np.isfinite(scratch)):
                    raise RuntimeError(error.value.decode() or "Nonfinite CUDA tallies")

                total += scratch
                self.provenance["gpu_dispatches"] += 1

            counters = (ctypes.c_uint64 * 6)()
            self._native.monki_cuda_counters(self._handle, counters)
            self.provenance["scatters"] = int(counters[0])
            self.provenance["photons"] = int(counters[4])
            self.provenance["kernel_launches"] = int(counters[5])

            if self.profile:
                self.provenance["gpu_seconds"] = self._native.monki_cuda_gpu_seconds(self._handle)

            results = []
            stokes_count = nmat * nx * ny * angles

            for request, values in zip(controls, total, strict=True):
                stokes = values[:stokes_count].reshape((nmat, nx, ny, angles), order="F").copy()
                paths = weights = None

                if self._paths:
                    path_count = nx * ny * nz * angles
                    paths = (
                        values[stokes_count : stokes_count + path_count]
                        .reshape((nx, ny, nz, angles), order="F")
                        .copy()
                    )
                    weights = (
                        values[stokes_count + path_count : stokes_count + path_count + nx * ny * angles]
                        .reshape((nx, ny, angles), order="F")
                        .copy()
                    )

                orders = None

                if self.orders:
                    at = stokes_count + ((nx * ny * nz * angles + nx * ny * angles) if self._paths else 0)
                    locations = nmat * nx * ny * nz * angles
                    orders = {
                        "single": values[at : at + stokes_count].reshape((nmat, nx, ny, angles), order="F").copy(),
                        "locations": values[at + stokes_count : at + stokes_count + locations]
                        .reshape((nmat, nx, ny, nz, angles), order="F")
                        .copy(),
                        "single_locations": values[at + stokes_count + locations :]
                        .reshape((nmat, nx, ny, nz, angles), order="F")
                        .copy(),
                    }

                results.append(RawTallies(request, stokes, paths, weights, orders))

            self._round = controls[-1].round_index
            return results
        except BaseException:
            self.close()
            raise
