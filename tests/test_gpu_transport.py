"""GPU parity: the sm_103a kernels through the C ABI against the CPU oracle.

Three levels, from exact to statistical:
  * helpers: Philox known answer and streams bit-exact; the polarization probe within
    rtol 1e-5 / atol 1e-7 (the tolerance of the reference's own probe test);
  * the FP64 transport build against the FP64 oracle on the same Philox streams: each
    tally within rtol 1e-6 of the oracle (rounding of libm and summation order only);
  * the FP32 product transport against the oracle with independent seeds: the reference
    criterion, |z| < 3 in at least 99 % of entries and mean z within 0.1 of zero.
"""

from __future__ import annotations

import ctypes
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _err():
    return ctypes.create_string_buffer(1024)


def test_gpu_philox_matches_published_known_answer(native, device):
    from monki.execution.native import U32P

    kat = json.loads((GOLDEN / "philox_kat.json").read_text())
    ctr = np.array(kat["counter"], dtype=np.uint32)
    key = np.array(kat["key"], dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    err = _err()
    assert native.monki_cuda_probe_philox(0, ctr.ctypes.data_as(U32P), key.ctypes.data_as(U32P), 1, out.ctypes.data_as(U32P), err, len(err)) == 0, err.value
    np.testing.assert_array_equal(out, kat["expected"])


def test_gpu_streams_equal_oracle_streams(native, device, oracle):
    from monki.execution.native import F32P, U32P

    rng = np.random.default_rng(1)
    counters = rng.integers(0, 2**32, size=(257, 4), dtype=np.uint64).astype(np.uint32)
    keys = rng.integers(0, 2**32, size=(257, 2), dtype=np.uint64).astype(np.uint32)
    out = np.zeros((257, 4), dtype=np.uint32)
    err = _err()
    status = native.monki_cuda_probe_philox(
        0, counters.ctypes.data_as(U32P), keys.ctypes.data_as(U32P), 257, out.ctypes.data_as(U32P), err, len(err)
    )
    assert status == 0, err.value

    for i in range(257):
        np.testing.assert_array_equal(out[i], oracle.philox(counters[i], keys[i]))

    draws = np.zeros(999, dtype=np.float32)
    assert native.monki_cuda_probe_uniforms(0, 12345, 77, 23274, 999, draws.ctypes.data_as(F32P), err, len(err)) == 0
    np.testing.assert_array_equal(draws.astype(np.float64), oracle.uniforms(12345, 77, 23274, 999))


@pytest.mark.parametrize("fp64", [0, 1])
def test_gpu_polarization_helpers_match_golden(native, device, fp64):
    from monki.execution.native import F64P

    probe = json.loads((GOLDEN / "polarization_probe.json").read_text())
    geometry = np.array(
        [[probe["incoming"][i], probe["outgoing"][i], probe["phi_in"][i], probe["phi_out"][i]] for i in range(3)]
    )
    stokes = np.array(probe["stokes"], dtype=np.float64)
    out = np.zeros((3, 3))
    err = _err()
    status = native.monki_cuda_probe_scatter_stokes(
        0, fp64, probe["depol"], geometry.ctypes.data_as(F64P), stokes.ctypes.data_as(F64P), 3, out.ctypes.data_as(F64P), err, len(err)
    )
    assert status == 0, err.value
    rtol, atol = (1e-12, 1e-14) if fp64 else (probe["rtol"], probe["atol"])
    np.testing.assert_allclose(out, np.array(probe["expected"]), rtol=rtol, atol=atol)


def _session(scene, precision="fp32", **kw):
    from monki.execution import CUDA

    backend = CUDA(precision=precision, **kw)
    backend.prepare(scene)
    return backend


def _controls(scene, rounds, seed, first_round=1):
    nmat, nx, ny, nz, angles = scene.shape
    per_round = scene.photons_per_column * nx * ny
    return [per_round * rounds, 0, first_round, seed, 100000, 0, per_round, rounds]


def _gpu_rounds(scene, rounds, seed, precision, **kw):
    from monki.execution import BatchControls

    with _session(scene, precision, seed=seed, **kw) as backend:
        batches = backend.run_batches([BatchControls(i, scene.photons_per_column) for i in range(1, rounds + 1)])
        return batches, dict(backend.provenance)


def _flat(batch):
    parts = [batch.stokes.ravel(order="F")]
    if batch.weighted_paths is not None:
        parts += [batch.weighted_paths.ravel(order="F"), batch.weights.ravel(order="F")]
    return np.concatenate(parts)


@pytest.mark.parametrize("engine", ["wavefront", "megakernel"])
@pytest.mark.parametrize("name", ["clear_sky", "layered_cloud", "box_cloud"])
def test_fp64_transport_reproduces_oracle_histories(oracle, device, name, engine):
    import monki.scenes as scenes

    builder = getattr(scenes, name)
    scene = builder(8, 2, nx=10, ny=8) if name != "box_cloud" else builder(8, 2, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))
    batches, provenance = _gpu_rounds(scene, 2, 23274, "fp64", engine=engine)
    expected, counters = oracle.run(scene.tables, _controls(scene, 2, 23274), 8)
    actual = np.stack([_flat(b) for b in batches])
    assert provenance["scatters"] == counters["scatters"]
    close = np.isclose(actual, expected, rtol=1e-6, atol=1e-12)
    assert close.mean() == 1.0, f"{(~close).sum()} of {close.size} tallies differ"


def _zscores(a_rounds, b_rounds):
    a, b = np.asarray(a_rounds), np.asarray(b_rounds)
    n = a.shape[0]
    ma, mb = a.mean(0), b.mean(0)
    sa, sb = a.std(0, ddof=1) / np.sqrt(n), b.std(0, ddof=1) / np.sqrt(n)
    se = np.hypot(sa, sb)
    mask = se > 0
    return (ma - mb)[mask] / se[mask]


@pytest.mark.parametrize("name", ["clear_sky", "layered_cloud", "box_cloud"])
def test_fp32_transport_agrees_with_oracle_within_combined_se(oracle, device, name):
    import monki.scenes as scenes

    builder = getattr(scenes, name)
    rounds = 32
    # Full 30 x 20 grids: the mean-z criterion needs many (nearly independent) pixels.
    scene = builder(12, rounds)
    batches, _ = _gpu_rounds(scene, rounds, 881, "fp32")
    gpu = np.stack([_flat(b) for b in batches])
    cpu, _ = oracle.run(scene.tables, _controls(scene, rounds, 23274), 16)
    z = _zscores(gpu, cpu)
    assert np.mean(np.abs(z) < 3) >= 0.99, np.sort(np.abs(z))[-10:]
    assert abs(np.mean(z)) < 0.1


def test_dispatch_chunking_and_shards_preserve_streams(device):
    import monki.scenes as scenes
    from monki.execution import BatchControls

    scene = scenes.layered_cloud(6, 1, nx=8, ny=6)
    results = []

    for settings in ({"photons_per_dispatch": 97, "tally_shards": 1}, {"tally_shards": 32, "pool": 1024}):
        with _session(scene, "fp64", **settings) as backend:
            results.append(backend.run_batch(BatchControls(1, 6)))

    np.testing.assert_allclose(_flat(results[0]), _flat(results[1]), rtol=1e-9, atol=1e-14)


def test_grouped_rounds_equal_sequential_rounds(device):
    import monki.scenes as scenes
    from monki.execution import BatchControls

    scene = scenes.clear_sky(5, 1, nx=6, ny=5)
    requests = [BatchControls(i, 5) for i in range(1, 8)]

    with _session(scene, "fp64") as grouped, _session(scene, "fp64") as sequential:
        a = grouped.run_batches(requests)
        b = [sequential.run_batch(r) for r in requests]
        assert grouped.provenance["gpu_dispatches"] == 1
        assert sequential.provenance["gpu_dispatches"] == 7

    for x, y in zip(a, b, strict=True):
        assert x.controls == y.controls
        np.testing.assert_allclose(x.stokes, y.stokes, rtol=1e-10, atol=1e-15)


def test_truncated_histories_fail_and_release_session(device):
    import monki.scenes as scenes
    from monki.execution import BatchControls

    backend = _session(scenes.clear_sky(5, 1, nx=4, ny=3), max_steps=1)

    with pytest.raises(RuntimeError, match="round rejected"):
        backend.run_batch(BatchControls(1, 5))

    assert backend._handle is None and backend.metadata is None


@pytest.mark.parametrize("layered", [False, True])
def test_step_counts_persist_across_paused_walks(device, layered):
    """A one-step walk budget pauses every walk after each cell step, so a history's step
    count must survive many launches (in the record block without layer paths, in its own
    array with them): a cap of 8 steps rejects the round, a cap of 100,000 does not."""

    import monki.scenes as scenes
    from monki.execution import BatchControls

    scene = scenes.layered_cloud(20, 1) if layered else scenes.box_cloud(20, 1)
    ppc = scene.photons_per_column
    backend = _session(scene, walk=1, max_steps=8, tail=0)
    with pytest.raises(RuntimeError, match="round rejected"):
        backend.run_batch(BatchControls(1, ppc))
    assert backend._handle is None

    backend = _session(scene, walk=1, max_steps=100_000, tail=0)
    batch = backend.run_batch(BatchControls(1, ppc))
    assert np.isfinite(batch.stokes).all() and batch.stokes[0].sum() > 0
    backend.close()


def test_invalid_device_does_not_fall_back(device):
    import monki.scenes as scenes
    from monki.execution import CUDA

    with CUDA(device=2**32 - 1) as backend:
        with pytest.raises(RuntimeError, match="unavailable"):
            backend.prepare(scenes.clear_sky(2, 1, nx=3, ny=2))
        assert backend._handle is None


def test_batch_validation_precedes_dispatch(device):
    import monki.scenes as scenes
    from monki.execution import BatchControls

    with _session(scenes.clear_sky(2, 1, nx=3, ny=2)) as backend:
        with pytest.raises(ValueError, match="sequential"):
            backend.run_batches([BatchControls(1, 2), BatchControls(3, 2)])
        assert backend.provenance["gpu_dispatches"] == 0
        assert backend.run_batch(BatchControls(1, 2)).controls.round_index == 1


@pytest.mark.parametrize("setting,value", [("seed", 1), ("save_path", False), ("tally_shards", 1), ("profile", True)])
def test_configuration_changes_require_reprepare(device, setting, value):
    import monki.scenes as scenes
    from monki.execution import BatchControls

    with _session(scenes.layered_cloud(2, 1, nx=3, ny=2)) as backend:
        setattr(backend, setting, value)
        with pytest.raises(ValueError, match="reprepare"):
            backend.run_batch(BatchControls(1, 2))
        assert backend.provenance["gpu_dispatches"] == 0


@pytest.mark.parametrize("name", ["layered_cloud", "box_cloud"])
def test_uniform_prefix_matches_explicit_detector_traversal(native, device, name):
    import monki.scenes as scenes
    from monki.execution.native import F64P

    builder = getattr(scenes, name)
    scene = builder(6, 1, nx=10, ny=8) if name != "box_cloud" else builder(6, 1, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))
    tables = np.ascontiguousarray(scene.tables)
    results = []

    for prefix in (1, 0):
        err = _err()
        handle = native.monki_cuda_create(0, tables.ctypes.data_as(F64P), tables.size, 1, f"precision=fp64,uniform_prefix={prefix}".encode(), err, len(err))
        assert handle, err.value
        try:
            count = int(native.monki_cuda_tally_count(handle))
            out = np.zeros(count)
            controls = (ctypes.c_uint32 * 8)(*_controls(scene, 1, 9))
            assert native.monki_cuda_run(handle, controls, out.ctypes.data_as(F64P), err, len(err)) == 0, err.value
            results.append(out)
        finally:
            native.monki_cuda_close(handle)

    np.testing.assert_allclose(results[0], results[1], rtol=1e-9, atol=1e-14)


@pytest.mark.parametrize("name", ["layered_cloud", "box_cloud", "wide_box"])
def test_rectangle_steps_match_face_by_face_walks(native, device, name):
    """Crossing an equal-extinction rectangle in one step is the face-by-face walk with the
    interior faces skipped: FP64 tallies agree to rounding, event counts exactly."""
    import monki.scenes as scenes
    from monki.execution.native import F64P, U64P

    if name == "wide_box":
        # A thin cloud in a wide clear field: long clear runs along both axes.
        scene = scenes.box_cloud(6, 1, nx=40, ny=24, box_x=(30, 33), box_y=(2, 22), optical_depth=5.0)
    elif name == "box_cloud":
        scene = scenes.box_cloud(6, 1, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))
    else:
        scene = scenes.layered_cloud(6, 1, nx=10, ny=8)
    tables = np.ascontiguousarray(scene.tables)
    results, scatters = [], []

    for rectangles in (1, 0):
        err = _err()
        handle = native.monki_cuda_create(0, tables.ctypes.data_as(F64P), tables.size, 1, f"precision=fp64,rectangles={rectangles}".encode(), err, len(err))
        assert handle, err.value
        try:
            count = int(native.monki_cuda_tally_count(handle))
            out = np.zeros(count)
            controls = (ctypes.c_uint32 * 8)(*_controls(scene, 1, 9))
            assert native.monki_cuda_run(handle, controls, out.ctypes.data_as(F64P), err, len(err)) == 0, err.value
            counters = np.zeros(6, dtype=np.uint64)
            native.monki_cuda_counters(handle, counters.ctypes.data_as(U64P))
            results.append(out)
            scatters.append(int(counters[0]))
        finally:
            native.monki_cuda_close(handle)

    assert scatters[0] == scatters[1]
    np.testing.assert_allclose(results[0], results[1], rtol=1e-9, atol=1e-14)


@pytest.mark.parametrize("name", ["layered_cloud", "box_cloud"])
def test_tail_launch_matches_launch_per_iteration(native, device, name):
    """Running a group's last photons to their ends in one launch (the tail kernel) is the
    same transport as three launches per iteration: equal event counts, and FP64 tallies
    within the oracle-parity tolerance (the kernels inline the same slot functions, but the
    compiler may contract their arithmetic differently, and rounding differences grow along
    a history that crosses a cloud edge)."""
    import monki.scenes as scenes
    from monki.execution.native import F64P, U64P

    scene = scenes.layered_cloud(6, 2, nx=10, ny=8) if name == "layered_cloud" else \
        scenes.box_cloud(6, 2, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))
    tables = np.ascontiguousarray(scene.tables)
    results = []

    for tail in (0, 1 << 20, 256):
        err = _err()
        config = f"precision=fp64,pool=4096,tail={tail}".encode()
        handle = native.monki_cuda_create(0, tables.ctypes.data_as(F64P), tables.size, 2, config, err, len(err))
        assert handle, err.value
        try:
            count = int(native.monki_cuda_tally_count(handle))
            out = np.zeros(2 * count)
            controls = (ctypes.c_uint32 * 8)(*_controls(scene, 2, 4))
            assert native.monki_cuda_run(handle, controls, out.ctypes.data_as(F64P), err, len(err)) == 0, err.value
            counters = np.zeros(6, dtype=np.uint64)
            native.monki_cuda_counters(handle, counters.ctypes.data_as(U64P))
            results.append((out, int(counters[0]), int(counters[4]), int(counters[5])))
        finally:
            native.monki_cuda_close(handle)

    (base, scatters, photons, launches), *others = results
    for out, s, p, n in others:
        assert (s, p) == (scatters, photons)
        assert n < launches  # the tail replaced launches
        np.testing.assert_allclose(out, base, rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("name", ["layered_cloud", "box_cloud"])
def test_fused_step_matches_separate_kernels(native, device, name):
    """Scattering each event and walking its photon on in one step kernel is the same
    transport as separate walk and scatter kernels: equal counts, FP64 tallies within the
    oracle-parity tolerance."""
    import monki.scenes as scenes
    from monki.execution.native import F64P, U64P

    scene = scenes.layered_cloud(6, 2, nx=10, ny=8) if name == "layered_cloud" else \
        scenes.box_cloud(6, 2, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))
    tables = np.ascontiguousarray(scene.tables)
    results = []
    for fused in (0, 1):
        err = _err()
        config = f"precision=fp64,pool=4096,tail=0,fused={fused}".encode()
        handle = native.monki_cuda_create(0, tables.ctypes.data_as(F64P), tables.size, 2, config, err, len(err))
        assert handle, err.value
        try:
            out = np.zeros(2 * int(native.monki_cuda_tally_count(handle)))
            controls = (ctypes.c_uint32 * 8)(*_controls(scene, 2, 8))
            assert native.monki_cuda_run(handle, controls, out.ctypes.data_as(F64P), err, len(err)) == 0, err.value
            counters = np.zeros(6, dtype=np.uint64)
            native.monki_cuda_counters(handle, counters.ctypes.data_as(U64P))
            results.append((out, int(counters[0]), int(counters[4])))
        finally:
            native.monki_cuda_close(handle)
    (a, sa, pa), (b, sb, pb) = results
    assert (sa, pa) == (sb, pb)
    np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-12)


def test_off_plane_polarization_is_nonzero_and_bounded(device):
    import monki.scenes as scenes

    scene = scenes.layered_cloud(20, 1, nx=6, ny=4)
    batches, _ = _gpu_rounds(scene, 1, 3, "fp32")
    stokes = batches[0].stokes
    assert np.max(np.abs(stokes[2])) > 1e-3 * np.max(stokes[0])
    assert np.all(np.hypot(stokes[1], stokes[2]) <= stokes[0] * 1.01 + 1e-12)


def test_group_ends_only_after_paused_walks_finish(native, oracle, device):
    """Photons paused by the per-launch walk budget are live: a round group must not end
    while one is still walking. Single-photon groups with a one-step budget pause at
    nearly every launch; each must reproduce the oracle's history."""
    import monki.scenes as scenes
    from monki.execution.native import F64P, U32P, U64P

    scene = scenes.box_cloud(8, 2, nx=12, ny=10, box_x=(3, 8), box_y=(2, 6))
    nmat, nx, ny, nz, angles = scene.shape
    per_round = 8 * nx * ny
    tables = np.ascontiguousarray(scene.tables)
    err = _err()
    handle = native.monki_cuda_create(0, tables.ctypes.data_as(F64P), tables.size, 2, b"precision=fp64,pool=1024,walk=1", err, len(err))
    assert handle, err.value
    try:
        count = native.monki_cuda_tally_count(handle)
        before = np.zeros(6, dtype=np.uint64)
        after = np.zeros(6, dtype=np.uint64)
        for photon in (99, 374, 5, 600):
            controls = np.array([1, photon, 1, 5, 100000, 0, per_round, 2], dtype=np.uint32)
            out = np.zeros(2 * count)
            native.monki_cuda_counters(handle, before.ctypes.data_as(U64P))
            status = native.monki_cuda_run(handle, controls.ctypes.data_as(U32P), out.ctypes.data_as(F64P), err, len(err))
            assert status == 0, err.value
            native.monki_cuda_counters(handle, after.ctypes.data_as(U64P))
            expected, counters = oracle.run(tables, controls, 1)
            assert int(after[0] - before[0]) == counters["scatters"], photon
            np.testing.assert_allclose(out, expected.ravel(), rtol=1e-6, atol=1e-12)
    finally:
        native.monki_cuda_close(handle)
