"""GPU Measurement Set column conversions against the oracle, bit for bit (the same IEEE
operations in the same order): ragged row/channel counts against the 32 x 32 transpose tiles, one
and four correlations, pageable and page-locked buffers, and the device-resident ingest of a DATA
block into an observation (FP64 and FP32 storage)."""
import ctypes as C

import numpy as np
import pytest

from radiolensfit2_gb300 import _lib, synth
import _oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    return _lib.load()


@pytest.fixture(scope="module")
def orc():
    return O.load_oracle()


PF, PD, PU8 = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_uint8)


def f(a):
    return a.ctypes.data_as(PF)


def d(a):
    return a.ctypes.data_as(PD)


def u8(a):
    return a.ctypes.data_as(PU8)


def pinned(a):
    torch = pytest.importorskip("torch")
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()


@pytest.mark.parametrize("rows,nch,npol,pin", [(1, 1, 1, False), (37, 3, 4, False), (1000, 17, 4, False),
                                                (4099, 33, 1, False), (200003, 16, 4, False),
                                                (200003, 16, 4, True)])
def test_read_vis_flags(lib, orc, rows, nch, npol, pin):
    rng = np.random.default_rng(rows + nch + npol)
    block = rng.standard_normal(rows * nch * npol * 2).astype(np.float32)
    fl = (rng.random(rows * nch * npol) < 0.1).astype(np.uint8)
    ref = np.zeros(rows * nch, np.complex128)
    orc.orc_ms_read_vis(O.fp(block), rows, nch, npol, O.cp(ref))
    fref = np.zeros(rows * nch, np.uint8)
    nref = orc.orc_ms_read_flag(O.bp(fl), rows, nch, npol, O.bp(fref))
    if pin:
        block, fl = pinned(block), pinned(fl)
    vis = pinned(np.zeros(rows * nch, np.complex128)) if pin else np.zeros(rows * nch, np.complex128)
    assert lib.rlf_ms_read_vis(f(block), rows, nch, npol, d(vis.view(np.float64))) == 0
    assert np.array_equal(vis, ref)
    out = np.zeros(rows * nch, np.uint8)
    n = lib.rlf_ms_read_flag(u8(fl), rows, nch, npol, u8(out))
    assert n == nref and np.array_equal(out, fref)


def test_coords_sigma_write(lib, orc):
    rng = np.random.default_rng(3)
    rows, nch = 70001, 5
    uvw = rng.uniform(-8000, 8000, rows * 3)
    u1, v1, w1 = np.zeros(rows), np.zeros(rows), np.zeros(rows)
    u2, v2, w2 = np.zeros(rows), np.zeros(rows), np.zeros(rows)
    l1 = orc.orc_ms_read_coords(O.dp(uvw), rows, O.dp(u1), O.dp(v1), O.dp(w1))
    l2 = lib.rlf_ms_read_coords(d(uvw), rows, d(u2), d(v2), d(w2))
    assert l1 == l2 and np.array_equal(u1, u2) and np.array_equal(v1, v2) and np.array_equal(w1, w2)
    sig = rng.uniform(-1, 3, rows * 4).astype(np.float32)
    s1, s2 = np.zeros(rows * nch, np.float32), np.zeros(rows * nch, np.float32)
    orc.orc_ms_read_sigma2(O.fp(sig), rows, nch, np.float32(2.5), O.fp(s1))
    assert lib.rlf_ms_read_sigma2(f(sig), rows, nch, np.float32(2.5), f(s2)) == 0
    assert np.array_equal(s1, s2)
    assert lib.rlf_ms_read_sigma2(None, rows, nch, np.float32(2.5), f(s2)) == 0
    assert np.all(s2 == np.float32(2.5))
    vis = rng.standard_normal(rows * nch) + 1j * rng.standard_normal(rows * nch)
    o1, o2 = np.zeros(rows * nch * 2, np.float32), np.zeros(rows * nch * 2, np.float32)
    orc.orc_ms_write_vis(O.cp(vis), rows, nch, O.fp(o1))
    assert lib.rlf_ms_write_vis(d(vis.view(np.float64)), rows, nch, f(o2)) == 0
    assert np.array_equal(o1, o2)


@pytest.mark.parametrize("precision", [_lib.RLF_F64, _lib.RLF_MIXED])
def test_obs_set_data_ms(lib, orc, precision):
    obs = synth.make_observation(n_ant=24, ha_hours=2.0, dt_s=600.0, n_ch=6)
    rng = np.random.default_rng(11)
    npol = 4
    block = rng.standard_normal(obs.n_rows * obs.n_ch * npol * 2).astype(np.float32)
    ref = np.zeros(obs.n_vis, np.complex128)
    orc.orc_ms_read_vis(O.fp(block), obs.n_rows, obs.n_ch, npol, O.cp(ref))
    from radiolensfit2_gb300.pipeline import DeviceObservation
    dev = DeviceObservation(obs, precision=precision)
    dev.set_data_ms(block.view(np.complex64), npol)
    data, _ = dev.get_vis()
    dev.close()
    if precision == _lib.RLF_F64:
        assert np.array_equal(data, ref)
    else:
        assert np.array_equal(data, ref.astype(np.complex64).astype(np.complex128))
