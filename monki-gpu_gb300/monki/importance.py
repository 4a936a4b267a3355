"""Learned detector importance for guided transport.

A small BF16 network (48 features -> 256 -> 256 -> 256 -> 1, GELU) maps each cell's
local optical properties, its column context and the sun/view geometry to the log of the
cell's detector importance: the mean Stokes-I peel-off contribution, per unit photon
weight, of an event in the cell and of the next seven events of its history. The
targets are the importance tallies the analog kernels produce (``CUDA(importance=True)``);
the network is trained and evaluated on the GB300 by hand-written tcgen05 kernels
(``csrc/mlp.cu``), and its prediction becomes the per-cell Russian-roulette scale of the
guided transport (``CUDA.set_roulette_scale``). The roulette keeps the estimator
unbiased whatever the network predicts; the prediction only moves the variance and cost.
"""

from __future__ import annotations

import ctypes
import math
import time
from dataclasses import dataclass

import numpy as np

from .execution import native as _native
from .guided import Guided

FEATURES = 48
# Guided transport under the learned weight window: Russian roulette below the cell's weight
# W = roulette x scale[cell], splitting above split x W. The window is the best constant one
# (roulette 0.25, split 2) moved per cell by the network, (importance / median) ** -0.25
# clipped to [0.85, 1.2]: on held-out box clouds it matches the constant window on the worst
# pixel's variance x cost (1.01x) and gains 2 % on the median pixel; stronger moves
# (exponent 0.5, [1, 2]) gain 23 % on the median pixel and lose 9 % on the worst. On a
# roulette-0.35 window the network's move ([0.7, 1.4]) gains 6-14 % on the worst pixel.
LEARNED_GUIDE = Guided(0.0, 0.25, 0.0, 2.0)
LEARNED_WINDOW = {"exponent": 0.25, "low": 0.85, "high": 1.2}
PARAMETERS = 64 * 256 + 256 + 2 * (256 * 256 + 256) + 256 + 1


# ------------------------------------------------------------------------------------
# Table stream parsing (transport.bin v1/v2 layout, kernels/cpu/worker.f90:1102-1120).
# ------------------------------------------------------------------------------------
@dataclass
class Tables:
    nx: int
    ny: int
    nz: int
    nmat: int
    angles: int
    species: int
    xunit: float
    yunit: float
    vartheta0: float
    phi0: float
    zunit: np.ndarray
    view_zenith: np.ndarray
    view_azimuth: np.ndarray
    albedo: np.ndarray  # (nx, ny)
    beta: np.ndarray  # (nx, ny, nz)
    fractions: np.ndarray  # (species + 1, nx, ny, nz)
    ssalb_gas: np.ndarray  # (nz,)
    ssalb: np.ndarray  # (species,)
    asymmetry: np.ndarray  # (species,) mean scattering cosine of each phase function


def parse_tables(tables) -> Tables:
    t = np.asarray(tables, dtype=np.float64)
    version, nx, ny, nz, nmat, angles, species = (int(v) for v in t[:7])
    at = 12
    xunit, yunit, _, vartheta0, phi0, phi = t[at : at + 6]
    at += 6

    def take(n):
        nonlocal at
        out = t[at : at + n]
        at += n
        return out

    zunit = take(nz).copy()
    view_zenith = take(angles).copy()
    view_azimuth = take(angles).copy() if version == 2 else np.full(angles, phi)
    take(nx * ny)
    albedo = take(nx * ny).reshape((nx, ny), order="F").copy()
    take(nx * ny)
    beta = take(nx * ny * nz).reshape((nx, ny, nz), order="F").copy()
    fractions = take((species + 1) * nx * ny * nz).reshape((species + 1, nx, ny, nz), order="F").copy()
    ssalb_gas = take(nz).copy()
    ssalb, asymmetry = [], []

    for _ in range(species):
        n, albedo_s = take(2)
        n = int(n)
        cosines, cdf, f11 = take(n), take(n), take(n)
        take(3 * n)
        ssalb.append(albedo_s)
        # Mean scattering cosine: trapezoid integral of mu F11 over the normalisation.
        norm = np.trapezoid(f11, cosines)
        asymmetry.append(float(np.trapezoid(cosines * f11, cosines) / norm) if norm > 0 else 0.0)

    return Tables(nx, ny, nz, nmat, angles, species, float(xunit), float(yunit), float(vartheta0), float(phi0),
                  zunit, view_zenith, view_azimuth, albedo, beta, fractions, ssalb_gas,
                  np.asarray(ssalb), np.asarray(asymmetry))


# ------------------------------------------------------------------------------------
# Features: 48 per cell, in Fortran cell order (i fastest, then j, then k).
# ------------------------------------------------------------------------------------
def cell_features(tables) -> np.ndarray:
    """Feature matrix (nx * ny * nz, 48) of float32.

    local (8)      log10 extinction, single-scattering albedo, asymmetry, gas and
                   particle fractions (3), altitude / 60 km, thickness
    column (16)    log(1 + optical depth) above, below and in total; above in the eight
                   neighbouring columns; particle optical depth above and below; log10 of
                   the column's largest extinction; surface albedo; layer index / nz
    geometry (12)  cos and sin of the solar zenith; per view cos VZA and sin VZA times
                   cos / sin of the relative azimuth; one zero
    paths (12)     per view log(1 + tau_above / mu_v) and exp(-tau_above / mu_v); the same
                   two along the sun; tau below / mu0; per view the cosine of the angle
                   between the solar propagation and the view direction
    """

    t = parse_tables(tables) if not isinstance(tables, Tables) else tables
    nx, ny, nz = t.nx, t.ny, t.nz
    dz = t.zunit[None, None, :]
    tau = t.beta * dz  # (nx, ny, nz)
    above = np.cumsum(tau[:, :, ::-1], axis=2)[:, :, ::-1] - tau  # strictly above the cell
    below = np.cumsum(tau, axis=2) - tau
    total = tau.sum(axis=2, keepdims=True)
    particle_tau = (t.fractions[:-1].sum(axis=0) if t.species else np.zeros_like(tau)) * tau
    p_above = np.cumsum(particle_tau[:, :, ::-1], axis=2)[:, :, ::-1] - particle_tau
    p_below = np.cumsum(particle_tau, axis=2) - particle_tau
    ssa = t.fractions[-1] * t.ssalb_gas[None, None, :]
    g = np.zeros_like(tau)

    for s in range(t.species):
        ssa = ssa + t.fractions[s] * t.ssalb[s]
        g = g + t.fractions[s] * t.asymmetry[s]

    frac = np.zeros((3, nx, ny, nz))
    frac[0] = t.fractions[-1]
    for s in range(min(t.species, 2)):
        frac[1 + s] = t.fractions[s]
    heights = np.concatenate([[0.0], np.cumsum(t.zunit)])
    centre = 0.5 * (heights[:-1] + heights[1:])
    k_index = np.arange(nz)
    f = []
    f.append(np.log10(t.beta + 1e-6))
    f.append(ssa)
    f.append(g)
    f.extend(frac)
    f.append(np.broadcast_to(centre / 60.0, (nx, ny, nz)))
    f.append(np.broadcast_to(t.zunit, (nx, ny, nz)))
    f.append(np.log1p(above))
    f.append(np.log1p(below))
    f.append(np.broadcast_to(np.log1p(total), (nx, ny, nz)))
    for di, dj in ((1, 0), (-1, 0), (0, 1), (0, -1), (1, 1), (1, -1), (-1, 1), (-1, -1)):
        f.append(np.log1p(np.roll(np.roll(above, -di, axis=0), -dj, axis=1)))
    f.append(np.log1p(p_above))
    f.append(np.log1p(p_below))
    f.append(np.broadcast_to(np.log10(t.beta.max(axis=2, keepdims=True) + 1e-6), (nx, ny, nz)))
    f.append(np.broadcast_to(t.albedo[:, :, None], (nx, ny, nz)))
    f.append(np.broadcast_to(k_index / nz, (nx, ny, nz)))
    sza = math.radians(180.0 - t.vartheta0)
    mu0 = max(abs(math.cos(sza)), 1e-3)
    geometry = [math.cos(sza), math.sin(sza)]
    paths = []
    sun = np.array([math.sin(math.radians(t.vartheta0)) * math.cos(math.radians(t.phi0)),
                    math.sin(math.radians(t.vartheta0)) * math.sin(math.radians(t.phi0)),
                    math.cos(math.radians(t.vartheta0))])
    views = []

    for v in range(3):
        vz = math.radians(t.view_zenith[v % t.angles])
        raa = math.radians(t.view_azimuth[v % t.angles] - t.phi0)
        geometry += [math.cos(vz), math.sin(vz) * math.cos(raa), math.sin(vz) * math.sin(raa)]
        mu = max(math.cos(vz), 1e-3)
        paths += [np.log1p(above / mu), np.exp(-above / mu)]
        az = math.radians(t.view_azimuth[v % t.angles])
        views.append(np.array([math.sin(vz) * math.cos(az), math.sin(vz) * math.sin(az), math.cos(vz)]))

    geometry.append(0.0)
    paths += [np.log1p(above / mu0), np.exp(-above / mu0), np.log1p(below / mu0)]
    paths += [np.full((nx, ny, nz), float(sun @ d)) for d in views]
    f.extend(np.broadcast_to(v, (nx, ny, nz)) for v in geometry)
    f.extend(paths)
    stacked = np.stack([np.asarray(a, dtype=np.float64) for a in f], axis=-1)  # nx, ny, nz, 48
    assert stacked.shape[-1] == FEATURES, stacked.shape
    return np.ascontiguousarray(stacked.transpose(2, 1, 0, 3).reshape(-1, FEATURES), dtype=np.float32)


def importance_targets(tally, minimum_events: int = 16, floor: float = 1e-8):
    """log mean importance per cell and a weight (0 for cells with too few events), both
    (nx * ny * nz,) in Fortran cell order, from a tally of shape (2, nx, ny, nz)."""

    sums, counts = np.asarray(tally[0]), np.asarray(tally[1])
    mean = np.divide(sums, counts, out=np.zeros_like(sums), where=counts > 0)
    target = np.log(mean + floor)
    weight = np.where(counts >= minimum_events, np.minimum(1.0, counts / (4.0 * minimum_events)), 0.0)
    flat = lambda a: np.ascontiguousarray(a.ravel(order="F"), dtype=np.float32)  # noqa: E731
    return flat(target), flat(weight)


def roulette_scale(log_importance, shape, *, exponent: float = 0.5, low: float = 0.5, high: float = 2.0):
    """Per-cell roulette scale (nx, ny, nz) from predicted log importance: cells more
    important than the median get a lower roulette weight (fewer photons killed there) and
    less important ones a higher one, (importance / median) ** -exponent clipped to
    [low, high]."""

    values = np.asarray(log_importance, dtype=np.float64).reshape(shape, order="F")
    reference = np.median(values)
    return np.clip(np.exp(-exponent * (values - reference)), low, high)


# ------------------------------------------------------------------------------------
# The network on the GPU.
# ------------------------------------------------------------------------------------
class ImportanceModel:
    """The importance network, resident on one GB300 (tcgen05 training and inference).

    ``rows`` bounds a training minibatch and an inference pass (larger inputs run in
    passes). Parameters are FP32 masters (``params``); the kernels use BF16 copies.
    """

    def __init__(self, device: int = 0, *, rows: int = 65536, seed: int = 0, params=None, library=None):
        self._native = _native.load(library or _native.LIBRARY)
        if int(self._native.monki_mlp_param_count()) != PARAMETERS:
            raise RuntimeError("Rebuild the CUDA library: network layout mismatch")
        error = ctypes.create_string_buffer(4096)
        self._handle = self._native.monki_mlp_create(device, FEATURES, rows, seed, error, len(error))
        if not self._handle:
            raise RuntimeError(error.value.decode() or "network creation failed")
        self.rows = rows
        if params is None:
            params = initial_params(seed)
        self.params = params
        # Input standardisation, set by the first fit (identity before).
        self.mean = np.zeros(FEATURES, dtype=np.float32)
        self.scale = np.ones(FEATURES, dtype=np.float32)

    def _standard(self, features):
        x = np.asarray(features, dtype=np.float32)
        if x.ndim != 2 or x.shape[1] != FEATURES:
            raise ValueError(f"features must have shape (rows, {FEATURES})")
        return np.ascontiguousarray((x - self.mean) * self.scale, dtype=np.float32)

    def _check(self, status, error):
        if status:
            raise RuntimeError(error.value.decode() or "network call failed")

    @property
    def params(self) -> np.ndarray:
        out = np.zeros(PARAMETERS, dtype=np.float32)
        error = ctypes.create_string_buffer(4096)
        self._check(self._native.monki_mlp_get_params(self._handle, out.ctypes.data_as(_native.F32P), out.size, error, len(error)), error)
        return out

    @params.setter
    def params(self, values) -> None:
        values = np.ascontiguousarray(values, dtype=np.float32)
        if values.shape != (PARAMETERS,):
            raise ValueError(f"expected {PARAMETERS} parameters")
        error = ctypes.create_string_buffer(4096)
        self._check(self._native.monki_mlp_set_params(self._handle, values.ctypes.data_as(_native.F32P), values.size, error, len(error)), error)

    def predict(self, features) -> np.ndarray:
        x = self._standard(features)
        y = np.zeros(x.shape[0], dtype=np.float32)
        error = ctypes.create_string_buffer(4096)
        self._check(self._native.monki_mlp_forward(self._handle, x.ctypes.data_as(_native.F32P), x.shape[0],
                                                   y.ctypes.data_as(_native.F32P), error, len(error)), error)
        return y

    def gradients(self, features, target, weight):
        """(loss, gradient) of one batch: loss = sum w (y - t)^2 / sum w."""

        x = self._standard(features)
        t = np.ascontiguousarray(target, dtype=np.float32)
        w = np.ascontiguousarray(weight, dtype=np.float32)
        g = np.zeros(PARAMETERS, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        error = ctypes.create_string_buffer(4096)
        self._check(self._native.monki_mlp_gradients(self._handle, x.ctypes.data_as(_native.F32P), t.ctypes.data_as(_native.F32P),
                                                     w.ctypes.data_as(_native.F32P), x.shape[0], g.ctypes.data_as(_native.F32P),
                                                     loss.ctypes.data_as(_native.F32P), error, len(error)), error)
        return float(loss[0]), g

    def fit(self, features, target, weight, *, steps: int, batch: int, learning_rate: float = 1e-3) -> np.ndarray:
        """Adam on minibatches drawn on the device; returns the per-step losses. The first
        fit also fixes the input standardisation (mean and spread of each feature)."""

        raw = np.asarray(features, dtype=np.float32)
        if not np.any(self.mean) and np.all(self.scale == 1.0):
            self.mean = raw.mean(axis=0).astype(np.float32)
            spread = raw.std(axis=0)
            self.scale = np.where(spread > 1e-6, 1.0 / np.maximum(spread, 1e-6), 1.0).astype(np.float32)
        x = self._standard(raw)
        t = np.ascontiguousarray(target, dtype=np.float32)
        w = np.ascontiguousarray(weight, dtype=np.float32)
        error = ctypes.create_string_buffer(4096)
        self._check(self._native.monki_mlp_set_data(self._handle, x.ctypes.data_as(_native.F32P), t.ctypes.data_as(_native.F32P),
                                                    w.ctypes.data_as(_native.F32P), x.shape[0], error, len(error)), error)
        losses = np.zeros(steps, dtype=np.float32)
        start = time.perf_counter()
        self._check(self._native.monki_mlp_train(self._handle, steps, batch, learning_rate,
                                                 losses.ctypes.data_as(_native.F32P), error, len(error)), error)
        self.fit_seconds = time.perf_counter() - start
        return losses

    def close(self) -> None:
        if getattr(self, "_handle", None):
            self._native.monki_mlp_close(self._handle)
            self._handle = None

    def __enter__(self):
        return self

    def __exit__(self, *args):
        self.close()

    def __del__(self):
        self.close()


def initial_params(seed: int = 0, features: int = FEATURES) -> np.ndarray:
    """He-uniform hidden layers (zero weights on the padded inputs), a small output layer."""

    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, shape in ((features, (256, 64)), (256, (256, 256)), (256, (256, 256))):
        bound = math.sqrt(6.0 / fan_in)
        w = rng.uniform(-bound, bound, size=shape)
        if shape[1] == 64:
            w[:, features:] = 0.0
        parts += [w.ravel(), np.zeros(256)]
    parts += [rng.uniform(-1.0, 1.0, size=256) / 16.0, np.zeros(1)]
    return np.concatenate(parts).astype(np.float32)


def pilot(scene, device: int = 0, rounds: int = 2, photons_per_column: int | None = None, seed: int = 7,
          pixel_weights=None):
    """Importance tally of a short analog run, shape (2, nx, ny, nz); contributions are
    weighted per output pixel by ``pixel_weights`` (nx, ny, angles) when given."""

    from .execution import CUDA, BatchControls

    ppc = photons_per_column or scene.photons_per_column
    with CUDA(device=device, seed=seed, importance=True) as backend:
        backend.prepare(scene)
        if pixel_weights is not None:
            backend.set_importance_weights(pixel_weights)
        batches = backend.run_batches([BatchControls(i, ppc) for i in range(1, rounds + 1)])
        tally = backend.importance()
    return tally, batches


def objective_weights(batches, photons_per_column: int, power: float = 2.0):
    """Per-pixel weights (nx, ny, angles) for the precision target SE/|I| < r in every
    pixel and view: (relative error / the largest relative error) ** power from the
    rounds of a pilot, so contributions to the pixels that set the time count most."""

    intensity = np.stack([b.stokes[0] for b in batches]) / photons_per_column
    mean = intensity.mean(axis=0)
    spread = intensity.std(axis=0, ddof=1) if len(batches) > 1 else np.abs(mean)
    relative = np.divide(spread, np.abs(mean), out=np.zeros_like(mean), where=np.abs(mean) > 0)
    top = relative.max()
    return (relative / top) ** power if top > 0 else np.ones_like(mean)


# ------------------------------------------------------------------------------------
# Training set, training and evaluation.
# ------------------------------------------------------------------------------------
def relative_weights(batches, photons_per_column: int, low: float = 0.1, high: float = 10.0):
    """Per-pixel weights (nx, ny, angles) for a target on the relative error of every pixel
    and view: the domain-mean intensity over the pixel's own, clipped to [low, high], so a
    unit of a dark pixel's intensity counts as much as the same fraction of a bright one."""

    intensity = np.mean([b.stokes[0] for b in batches], axis=0) / photons_per_column
    mean = float(np.mean(np.abs(intensity)))
    ratio = np.divide(mean, np.abs(intensity), out=np.full_like(intensity, high), where=np.abs(intensity) > 0)
    return np.clip(ratio, low, high)


def objective_tally(scene, *, objective: str = "relative", device: int = 0, rounds: int = 2,
                    photons_per_column: int = 300, seed: int = 7):
    """The importance tally of a pilot for a precision objective: "relative" weights the
    contributions per pixel by ``relative_weights`` of a one-round analog pre-pilot (the
    target is every pixel's relative error); "total" leaves them unweighted (the summed
    intensity)."""

    if objective not in ("relative", "total"):
        raise ValueError("objective must be 'relative' or 'total'")
    weights = None
    if objective == "relative":
        _, first = pilot(scene, device=device, rounds=1, photons_per_column=photons_per_column, seed=seed + 1)
        weights = relative_weights(first, photons_per_column)
    tally, _ = pilot(scene, device=device, rounds=rounds, photons_per_column=photons_per_column, seed=seed,
                     pixel_weights=weights)
    return tally


def training_rows(scene, *, device: int = 0, rounds: int = 2, photons_per_column: int = 300, seed: int = 7,
                  limit: int = 40000, rng=None, objective: str = "relative"):
    """(features, target, weight) of the cells of one scene with enough pilot events, at
    most ``limit`` of them (drawn at random), for ``objective`` (see objective_tally)."""

    tally = objective_tally(scene, objective=objective, device=device, rounds=rounds,
                            photons_per_column=photons_per_column, seed=seed)
    target, weight = importance_targets(tally)
    keep = np.flatnonzero(weight > 0)
    if keep.size > limit:
        keep = (rng or np.random.default_rng(seed)).choice(keep, size=limit, replace=False)
    features = cell_features(scene.tables)
    return features[keep], target[keep], weight[keep]


def r_squared(prediction, target, weight) -> float:
    """Weighted coefficient of determination of a prediction."""

    w = np.asarray(weight, dtype=np.float64)
    t = np.asarray(target, dtype=np.float64)
    mean = np.sum(w * t) / np.sum(w)
    residual = np.sum(w * (np.asarray(prediction) - t) ** 2)
    total = np.sum(w * (t - mean) ** 2)
    return float(1.0 - residual / total) if total > 0 else 0.0


def training_scenes(count: int = 24):
    """The training family: scenes of the batched generator (seeds 10000 on, photons
    scaled down) and box clouds placed at random (seeds 2000 on, disjoint from the
    held-out box-cloud seeds 1000-1015)."""

    from . import scenes

    return [scenes.batched_scene(10000 + s, photons_scale=0.01) for s in range(count)] + [
        scenes.box_cloud_variant(2000 + s, 300, 2) for s in range(count)
    ]


def train_model(training, *, device: int = 0, steps: int = 3000, batch: int = 65536, learning_rate: float = 1e-3,
                photons_per_column: int = 300, rows_per_scene: int = 20000, seed: int = 1, objective: str = "relative"):
    """Pilot every training scene, then train a network on the device. Returns
    (model, per-step losses, training rows)."""

    rng = np.random.default_rng(seed)
    parts = [training_rows(scene, device=device, photons_per_column=photons_per_column, limit=rows_per_scene, rng=rng,
                           objective=objective)
             for scene in training]
    x = np.concatenate([p[0] for p in parts])
    t = np.concatenate([p[1] for p in parts])
    w = np.concatenate([p[2] for p in parts])
    model = ImportanceModel(device, rows=batch, seed=seed)
    losses = model.fit(x, t, w, steps=steps, batch=batch, learning_rate=learning_rate)
    return model, losses, len(t)


def learned_scale(model, scene, **transform):
    """The roulette scale (nx, ny, nz) a trained network gives a scene (the window of
    LEARNED_WINDOW unless ``transform`` overrides it)."""

    _, nx, ny, nz, _ = scene.shape
    return roulette_scale(model.predict(cell_features(scene.tables)), (nx, ny, nz), **{**LEARNED_WINDOW, **transform})


def main(argv=None) -> int:
    """``python -m monki.importance``: pilot the training family, train the network on the
    GPU and report the fit; ``--out`` keeps its parameters and input standardisation."""

    import argparse

    parser = argparse.ArgumentParser(prog="python -m monki.importance")
    parser.add_argument("--scenes", type=int, default=24, help="training scenes of each family")
    parser.add_argument("--steps", type=int, default=3000)
    parser.add_argument("--batch", type=int, default=65536)
    parser.add_argument("--objective", choices=("relative", "total"), default="relative")
    parser.add_argument("--device", type=int, default=0)
    parser.add_argument("--out", default=None, help="write params, mean and scale to this .npz")
    args = parser.parse_args(argv)
    start = time.perf_counter()
    model, losses, rows = train_model(training_scenes(args.scenes), device=args.device, steps=args.steps,
                                      batch=args.batch, objective=args.objective)
    with model:
        flops = len(losses) * model.rows * 2 * (3 * (64 * 256 + 2 * 256 * 256) - 64 * 256)
        print(f"rows {rows}; steps {len(losses)} at batch {model.rows}; loss {losses[:20].mean():.4f} -> "
              f"{losses[-50:].mean():.4f}; fit {model.fit_seconds:.3f} s ({flops / model.fit_seconds / 1e12:.1f} TFLOP/s "
              f"of GEMM work); with pilots {time.perf_counter() - start:.1f} s")
        if args.out:
            np.savez(args.out, params=model.params, mean=model.mean, scale=model.scale)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
