"""Host logic of the CUDA backend over a fake of its C ABI, on CPU.

The reference's Metal backend contract (python/monki/execution/metal.py:23-349, its device
tests tests/integration/test_metal.py:106-262): requests are validated before any device
work, rounds are sequential from one, consecutive equal rounds share a dispatch and come
back in order, a dispatch larger than the photon limit is chunked and summed, any native
failure closes the session, results are owned by the caller and outlive the session, a
settings change needs a new prepare, and close is idempotent. Here ``monki_cuda_*`` is a
Python fake that records every call and writes known tallies, so each rule is checked
without a GPU; the GPU tests check the same rules against the real library.
"""

from __future__ import annotations

import numpy as np
import pytest


class FakeNative:
    """Records calls; tally value of (round r, element e, dispatch first photon f) is
    1000 r + e + f / 1e6, so sums, order and chunking are visible in the results."""

    def __init__(self, fail_create=None, fail_run_at=None, nonfinite=False, count_offset=0):
        self.calls = []
        self.runs = []
        self.closed = []
        self.handles = 0
        self.fail_create = fail_create
        self.fail_run_at = fail_run_at
        self.nonfinite = nonfinite
        self.count_offset = count_offset
        self.count = 0

    def monki_cuda_create(self, device, tables, n, capacity, config, err, errlen):
        self.calls.append(("create", int(capacity), config))
        if self.fail_create:
            err.value = self.fail_create.encode()
            return None
        t = np.ctypeslib.as_array(tables, shape=(n,))
        nx, ny, nz, nmat, angles = (int(v) for v in t[1:6])
        self.count = nmat * nx * ny * angles + (nx * ny * (nz + 1) * angles if t[10] else 0) + self.count_offset
        self.handles += 1
        return self.handles

    def monki_cuda_tally_count(self, handle):
        return self.count

    def monki_cuda_device_name(self, handle):
        return b"fake"

    def monki_cuda_run(self, handle, command, out, err, errlen):
        words = list(command)
        self.runs.append(words)
        if self.fail_run_at is not None and len(self.runs) == self.fail_run_at:
            err.value = b"launch failed (flag 16: history cap)"
            return 16
        rounds = words[7]
        values = np.ctypeslib.as_array(out, shape=(rounds * self.count,)).reshape(rounds, self.count)
        for r in range(rounds):
            values[r] = 1000.0 * (words[2] + r) + np.arange(self.count) + words[1] / 1e6
        if self.nonfinite:
            values[0, 0] = np.nan
        return 0

    def monki_cuda_counters(self, handle, out):
        for i in range(6):
            out[i] = 7 * (i + 1)

    def monki_cuda_gpu_seconds(self, handle):
        return 0.25

    def monki_cuda_close(self, handle):
        self.closed.append(handle)


@pytest.fixture
def fake(monkeypatch, tmp_path):
    from monki.execution import native

    state = {"fake": FakeNative()}
    monkeypatch.setattr(native, "load", lambda path=None: state["fake"])
    library = tmp_path / "libfake.so"
    library.write_bytes(b"not a library")
    state["library"] = str(library)
    return state


def _backend(fake, **kwargs):
    from monki.execution import CUDA

    return CUDA(library=fake["library"], **kwargs)


def _scene(paths=False):
    from monki import scenes

    return scenes.layered_cloud(4, 1, nx=3, ny=2) if paths else scenes.clear_sky(4, 1, nx=3, ny=2)


def _expected(fake, round_index, first=0):
    return 1000.0 * round_index + np.arange(fake["fake"].count) + first / 1e6


def test_rounds_are_sequential_and_checked_before_any_dispatch(fake):
    from monki.execution import BatchControls

    with _backend(fake) as backend:
        backend.prepare(_scene())
        with pytest.raises(ValueError, match="sequential"):
            backend.run_batch(BatchControls(2, 4))
        assert fake["fake"].runs == []
        assert backend.run_batch(BatchControls(1, 4)).controls.round_index == 1
        with pytest.raises(ValueError, match="sequential"):
            backend.run_batch(BatchControls(3, 4))
        with pytest.raises(TypeError, match="BatchControls"):
            backend.run_batches([(2, 4)])
        assert backend.run_batch(BatchControls(2, 4)).controls.round_index == 2
        assert len(fake["fake"].runs) == 2


def test_consecutive_rounds_share_a_dispatch_and_keep_their_order(fake):
    from monki.execution import BatchControls

    with _backend(fake) as backend:
        backend.prepare(_scene())
        requests = [BatchControls(i, 4) for i in range(1, 6)] + [BatchControls(6, 8)]
        results = backend.run_batches(requests)
        runs = fake["fake"].runs
        # Rounds 1-5 (4 photons per column) in one dispatch, round 6 (8) in its own.
        assert [(w[0], w[1], w[2], w[6], w[7]) for w in runs] == [(5 * 24, 0, 1, 24, 5), (48, 0, 6, 48, 1)]
        assert [r.controls.round_index for r in results] == [1, 2, 3, 4, 5, 6]
        for r in results:
            flat = r.stokes.ravel(order="F")
            np.testing.assert_array_equal(flat, _expected(fake, r.controls.round_index)[: flat.size])
        assert backend.provenance["gpu_dispatches"] == 2
        assert backend.provenance["scatters"] == 7 and backend.provenance["kernel_launches"] == 42


def test_large_groups_are_chunked_by_photons_and_summed(fake):
    from monki.execution import BatchControls

    with _backend(fake, photons_per_dispatch=50) as backend:
        backend.prepare(_scene())
        result = backend.run_batch(BatchControls(1, 4))  # 24 photons per round: one chunk
        assert len(fake["fake"].runs) == 1
        fake["fake"].runs.clear()
        results = backend.run_batches([BatchControls(2, 4), BatchControls(3, 4)])
        # 48 photons fit one dispatch of 50: one call; a round of 60 photons needs two.
        assert len(fake["fake"].runs) == 1
        fake["fake"].runs.clear()
        big = backend.run_batch(BatchControls(4, 10))
        assert [(w[0], w[1]) for w in fake["fake"].runs] == [(50, 0), (10, 50)]
        flat = big.stokes.ravel(order="F")
        np.testing.assert_allclose(flat, (_expected(fake, 4, 0) + _expected(fake, 4, 50))[: flat.size], rtol=1e-15)
        assert result.controls.round_index == 1 and [r.controls.round_index for r in results] == [2, 3]


def test_native_failure_closes_the_session(fake):
    from monki.execution import BatchControls

    fake["fake"] = FakeNative(fail_run_at=2)
    backend = _backend(fake)
    backend.prepare(_scene())
    backend.run_batch(BatchControls(1, 4))
    with pytest.raises(RuntimeError, match="history cap"):
        backend.run_batch(BatchControls(2, 4))
    assert fake["fake"].closed == [1] and backend.metadata is None
    with pytest.raises(RuntimeError, match="prepared"):
        backend.run_batch(BatchControls(2, 4))
    backend.close()
    backend.close()
    assert fake["fake"].closed == [1]


def test_nonfinite_tallies_close_the_session(fake):
    from monki.execution import BatchControls

    fake["fake"] = FakeNative(nonfinite=True)
    backend = _backend(fake)
    backend.prepare(_scene())
    with pytest.raises(RuntimeError, match="Nonfinite"):
        backend.run_batch(BatchControls(1, 4))
    assert fake["fake"].closed == [1]


def test_results_are_owned_and_outlive_the_session(fake):
    from monki.execution import BatchControls

    backend = _backend(fake)
    backend.prepare(_scene(paths=True))
    first = backend.run_batch(BatchControls(1, 4))
    kept = first.stokes.copy(), first.weighted_paths.copy(), first.weights.copy()
    first.stokes[:] = -1.0
    second = backend.run_batch(BatchControls(2, 4))
    backend.close()
    assert np.all(second.stokes.ravel(order="F") == _expected(fake, 2)[: second.stokes.size])
    assert second.weighted_paths.shape == (3, 2, _scene(paths=True).shape[3], 3)
    assert second.weights.shape == (3, 2, 3)
    assert np.all(kept[0] >= 1000.0) and np.all(kept[1] > 0) and np.all(kept[2] > 0)


def test_settings_changes_need_a_new_prepare_and_reprepare_replaces_the_session(fake):
    from monki.execution import BatchControls

    backend = _backend(fake)
    backend.prepare(_scene())
    backend.seed = 99
    with pytest.raises(ValueError, match="reprepare"):
        backend.run_batch(BatchControls(1, 4))
    backend.prepare(_scene())
    assert fake["fake"].closed == [1]
    assert backend.run_batch(BatchControls(1, 4)).controls.round_index == 1
    assert fake["fake"].runs[-1][3] == 99
    backend.close()
    assert fake["fake"].closed == [1, 2]


def test_create_failure_raises_the_library_message(fake):
    fake["fake"] = FakeNative(fail_create="Requested CUDA device is unavailable")
    backend = _backend(fake)
    with pytest.raises(RuntimeError, match="unavailable"):
        backend.prepare(_scene())
    assert backend.metadata is None and fake["fake"].closed == []


def test_tally_layout_mismatch_closes_the_new_session(fake):
    fake["fake"] = FakeNative(count_offset=1)
    backend = _backend(fake)
    with pytest.raises(RuntimeError, match="layout"):
        backend.prepare(_scene())
    assert fake["fake"].closed == [1] and backend.metadata is None


def test_controls_words_carry_the_session_settings(fake):
    from monki.execution import BatchControls

    with _backend(fake, seed=4242, max_steps=777, profile=True) as backend:
        backend.prepare(_scene())
        backend.run_batch(BatchControls(1, 4))
        words = fake["fake"].runs[0]
        assert words == [24, 0, 1, 4242, 777, 1, 24, 1]
        assert backend.provenance["gpu_seconds"] == 0.25
        config = fake["fake"].calls[0][2].decode()
        assert "precision=fp32" in config and "engine=wavefront" in config


def test_missing_library_raises_and_nothing_falls_back(tmp_path):
    """The product has no CPU path: without the CUDA library prepare raises, and no module of
    the package imports the oracle (test infrastructure only)."""

    import re
    from pathlib import Path

    from monki.execution import CUDA

    backend = CUDA(library=str(tmp_path / "libmonki_cuda.so"))
    with pytest.raises(FileNotFoundError):
        backend.prepare(_scene())
    assert backend.metadata is None

    package = Path(__file__).resolve().parents[1] / "monki-gpu_gb300"
    pattern = re.compile(r"^\s*(from|import)\s+oracle\b|monki_oracle", re.MULTILINE)
    offenders = [str(p) for p in package.rglob("*") if p.suffix in (".py", ".cu", ".cuh", ".h", ".cpp")
                 and pattern.search(p.read_text(errors="ignore"))]
    assert offenders == []
