"""The learned-importance network on the GB300 against its CPU restatement.

* the tcgen05 GEMM (BF16 operands, FP32 accumulation in TMEM) against float64 products
  of the same BF16 values, plain and split-K;
* forward values and the loss gradient of every parameter against oracle/mlp.py, which
  rounds to BF16 where the kernels do (remaining differences: FP32 accumulation order
  and the last BF16 rounding of values near a rounding boundary);
* Adam training on the device reduces the loss of a learnable target.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(x):
    from oracle import mlp

    return np.ascontiguousarray(mlp.bf16(x).astype(np.float32).view(np.uint32) >> 16).astype(np.uint16)


@pytest.mark.parametrize("m, n, k, splits", [(300, 256, 256, 1), (128, 64, 64, 1), (1000, 16, 128, 1), (256, 256, 1024, 4), (77, 48, 192, 3)])
def test_tensor_core_gemm_matches_float64_products(native, device, m, n, k, splits):
    from monki.execution.native import F32P

    rng = np.random.default_rng(m + n + k)
    a, b = rng.normal(size=(m, k)), rng.normal(size=(n, k))
    abits, bbits = _bits(a), _bits(b)
    c = np.zeros((m, n), dtype=np.float32)
    err = ctypes.create_string_buffer(1024)
    u16 = ctypes.POINTER(ctypes.c_uint16)
    status = native.monki_mlp_gemm_probe(0, abits.ctypes.data_as(u16), bbits.ctypes.data_as(u16), m, n, k, splits,
                                         c.ctypes.data_as(F32P), err, len(err))
    assert status == 0, err.value
    from oracle import mlp

    expected = mlp.bf16(a) @ mlp.bf16(b).T
    np.testing.assert_allclose(c, expected, rtol=1e-4, atol=1e-4 * np.abs(expected).max())


def _batch(rows, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(rows, 48)).astype(np.float32)
    t = (np.sin(x[:, 0]) + 0.5 * x[:, 1] ** 2 - x[:, 2] * x[:, 3]).astype(np.float32)
    w = rng.uniform(0.5, 1.5, size=rows).astype(np.float32)
    return x, t, w


def test_forward_and_gradients_match_the_oracle(device):
    from monki.importance import ImportanceModel
    from oracle import mlp

    x, t, w = _batch(300, 1)
    with ImportanceModel(rows=512, seed=3) as model:
        params = model.params
        y = model.predict(x)
        loss, grads = model.gradients(x, t, w)
    y_ref, _ = mlp.forward(params, x)
    np.testing.assert_allclose(y, y_ref, rtol=2e-2, atol=2e-2 * np.abs(y_ref).max())
    loss_ref, grads_ref = mlp.gradients(params, x, t, w)
    assert loss == pytest.approx(loss_ref, rel=1e-2)
    at = 0
    for name, shape in mlp.SHAPES:
        size = int(np.prod(shape))
        g, r = grads[at : at + size].astype(np.float64), grads_ref[at : at + size]
        at += size
        error = np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-30)
        cosine = g @ r / max(np.linalg.norm(g) * np.linalg.norm(r), 1e-30)
        assert error < 2e-2 and cosine > 0.999, (name, error, cosine)


def test_training_on_the_device_reduces_the_loss(device):
    from monki.importance import ImportanceModel

    x, t, w = _batch(20000, 2)
    with ImportanceModel(rows=4096, seed=5) as model:
        initial = model.gradients(x[:4096], t[:4096], w[:4096])[0]
        losses = model.fit(x, t, w, steps=300, batch=4096, learning_rate=2e-3)
        final = model.gradients(x[:4096], t[:4096], w[:4096])[0]
    assert np.all(np.isfinite(losses))
    assert final < 0.2 * initial, (initial, final, losses[::50])
