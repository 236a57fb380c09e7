"""Mixed-precision observations store their rows in uv order; every host-facing path keeps the
caller's order: the visibility round trip (pinned and pageable host buffers), the complex64
setter, the Measurement Set DATA reader and the simulator's noise, whose realisation is keyed by
the caller's visibility index and so matches the FP64 observation (caller's order) to FP32
rounding."""
import numpy as np
import pytest

from radiolensfit2_gb300 import _lib, synth
from radiolensfit2_gb300.pipeline import DeviceObservation

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def obs():
    # more rows than one uv bin holds, ragged against warps and transpose tiles
    return synth.make_observation(n_ant=23, ha_hours=1.0, dt_s=300.0, n_ch=5)


def _f32(x):
    return (x.real.astype(np.float32).astype(np.float64) + 1j * x.imag.astype(np.float32).astype(np.float64))


def test_vis_round_trip(obs):
    rng = np.random.default_rng(7)
    n = obs.n_vis
    data = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    sky = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    dev = DeviceObservation(obs, precision=_lib.RLF_MIXED)
    dev.set_vis(data, sky)
    d, s = dev.get_vis()
    assert np.array_equal(d, _f32(data)) and np.array_equal(s, _f32(sky))
    # pinned host buffers take the direct path
    import torch
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    dp, sp = pin(data[::-1].copy()), pin(sky[::-1].copy())
    dev.set_vis(dp, sp)
    d, s = dev.get_vis()
    assert np.array_equal(d, _f32(data[::-1])) and np.array_equal(s, _f32(sky[::-1]))
    # complex64 setter
    c64 = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    dev.set_data_c64(c64)
    d, _ = dev.get_vis()
    assert np.array_equal(d, c64.astype(np.complex128))
    dev.close()


def test_ms_data_reader_order(obs):
    rng = np.random.default_rng(8)
    rows, nch = obs.n_rows, obs.n_ch
    block = (rng.standard_normal((rows, nch, 1)) + 1j * rng.standard_normal((rows, nch, 1))).astype(np.complex64)
    out = []
    for prec in (_lib.RLF_F64, _lib.RLF_MIXED):
        dev = DeviceObservation(obs, precision=prec)
        dev.set_data_ms(block, 1)
        out.append(dev.get_vis()[0])
        dev.close()
    # the reader's Stokes I in uJy, [ch][row]: the same in both layouts to FP32 rounding
    assert np.array_equal(out[1], _f32(out[0]))
    expect = (block[:, :, 0].astype(np.complex128) * 1e6).T.reshape(-1)
    assert np.allclose(out[0], expect, rtol=1e-12, atol=0)


def test_simulator_noise_keyed_by_caller_index(obs):
    cat = synth.make_catalogue(6, 30.0, 200.0)
    out = []
    for prec in (_lib.RLF_F64, _lib.RLF_MIXED):
        dev = DeviceObservation(obs, precision=prec)
        dev.simulate(cat, 900.0, seed=11)
        out.append(dev.get_vis()[0])
        dev.close()
    scale = np.max(np.abs(out[0]))
    assert np.max(np.abs(out[1] - out[0])) < 1e-5 * scale
