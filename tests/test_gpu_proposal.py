"""The learned proposal's CUDA kernels (tcgen05 tensor-core convolutions, head, loss, resampler)
against a PyTorch FP32 reference on the CPU (tests/_cnn_ref.py) that rounds to bf16 where the
device path does.  Tolerances: the device and the reference differ only in the order of FP32
sums, which can flip a bf16 rounding of an activation or a gradient (one bf16 ulp, 2^-8), so the
head's outputs agree to 1e-2 of their scale and every parameter block's gradient to 2e-2 in
norm (measured differences are printed)."""
import ctypes as C

import numpy as np
import pytest

from radiolensfit2_gb300 import _lib

import _cnn_ref as R

pytestmark = pytest.mark.gpu

U16P = C.POINTER(C.c_uint16)


def _f(a):
    return a.ctypes.data_as(_lib.PF)


def _i(a):
    return a.ctypes.data_as(_lib.PI)


def _images(rng, n):
    x = np.zeros((n, 64, 64, 4), np.float32)
    x[..., 0] = rng.standard_normal((n, 64, 64)) * 0.5
    x[..., 1] = rng.standard_normal((n, 64, 64)) * 0.5
    x[..., 2] = (rng.random((n, 64, 64)) < 0.8).astype(np.float32)
    x[..., 3] = rng.random((n, 64, 64))
    return R.f32_to_bf16_bits(x)


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


def test_param_layout(lib):
    _, n = R.param_blocks()
    assert lib.rlf_cnn_param_count() == n == 30980


@pytest.mark.parametrize("n", [3, 130])
def test_forward_and_gradients_against_torch(lib, n):
    rng = np.random.default_rng(4 + n)
    params = R.init_params(rng)
    imgs = _images(rng, n)
    tgt = np.stack([rng.uniform(-0.5, 0.5, n), rng.uniform(-0.5, 0.5, n), rng.normal(-0.5, 0.4, n)], 1).astype(np.float32)
    h = lib.rlf_cnn_create(256, n)
    assert h
    try:
        assert lib.rlf_cnn_set_params(h, _f(params)) == 0
        assert lib.rlf_cnn_set_images(h, 0, n, imgs.ctypes.data_as(U16P)) == 0
        assert lib.rlf_cnn_set_targets(h, 0, n, _f(tgt)) == 0
        idx = np.arange(n, dtype=np.int32)
        g = np.zeros_like(params)
        loss = np.zeros(1, np.float32)
        out = np.zeros((n, 4), np.float32)
        assert lib.rlf_cnn_grads(h, _i(idx), n, _f(g), _f(loss), _f(out)) == 0
        # prediction path (stored images, chunks of the batch) gives the same outputs
        out2 = np.zeros((n, 4), np.float32)
        assert lib.rlf_cnn_predict(h, 0, n, _f(out2)) == 0
    finally:
        lib.rlf_cnn_destroy(h)
    ref_out, ref_loss, ref_g = R.forward_backward(params, imgs, tgt)
    scale = np.max(np.abs(ref_out))
    d_out = np.max(np.abs(out - ref_out)) / scale
    print(f"n={n}: head outputs max |d| / scale {d_out:.2e}; loss {loss[0]:.6f} vs {ref_loss:.6f}")
    assert d_out < 1e-2
    assert np.array_equal(out, out2)
    assert abs(loss[0] - ref_loss) < 1e-2 * max(1.0, abs(ref_loss))
    blocks, _ = R.param_blocks()
    for kind, off, shape in blocks:
        size = int(np.prod(shape))
        a, b = g[off:off + size], ref_g[off:off + size]
        rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
        print(f"  {kind}{shape}: |dg| / |g| = {rel:.2e}")
        assert rel < 2e-2, (kind, shape, rel)


def test_training_reduces_loss(lib):
    """Adam steps on a fixed batch drive the loss down (the optimiser and the gradients agree in
    sign and scale)."""
    rng = np.random.default_rng(9)
    n = 64
    params = R.init_params(rng, scale=0.5)
    imgs = _images(rng, n)
    tgt = np.stack([rng.uniform(-0.3, 0.3, n), rng.uniform(-0.3, 0.3, n), rng.normal(-0.5, 0.3, n)], 1).astype(np.float32)
    h = lib.rlf_cnn_create(n, n)
    try:
        lib.rlf_cnn_set_params(h, _f(params))
        lib.rlf_cnn_set_images(h, 0, n, imgs.ctypes.data_as(U16P))
        lib.rlf_cnn_set_targets(h, 0, n, _f(tgt))
        idx = np.arange(n, dtype=np.int32)
        loss = np.zeros(1, np.float32)
        first = None
        for it in range(60):
            assert lib.rlf_cnn_train_step(h, _i(idx), n, 3e-3, _f(loss)) == 0
            first = loss[0] if first is None else first
        print(f"loss {first:.4f} -> {loss[0]:.4f}")
        assert loss[0] < first - 0.1
    finally:
        lib.rlf_cnn_destroy(h)
