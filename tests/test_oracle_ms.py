"""The oracle's Measurement Set column conversions (measurement_set.cpp:203-453 applied to column
blocks; the reference's own readers need casacore and do not build here, so this row's parity is
pinned only to the restatement) against an independent numpy statement of the same loops:
layouts, Stokes I from one or four correlations, Jy -> uJy, flags, the flat SIGMA read and the
driver's fallback to the theoretical variance."""
import numpy as np
import pytest

import _oracle as O


@pytest.fixture(scope="module")
def orc():
    return O.load_oracle()


def np_read_vis(block, rows, nch, npol):
    b = block.reshape(rows, nch, npol, 2).astype(np.float64)
    v = b[:, :, 0, :].copy()
    if npol == 4:
        v = (v + b[:, :, 3, :]) * 0.5
    v = v * 1e6
    return (v[..., 0] + 1j * v[..., 1]).T.reshape(-1)  # [ch][row]


@pytest.mark.parametrize("rows,nch,npol", [(1, 1, 1), (37, 3, 1), (37, 3, 4), (1000, 17, 4), (64, 32, 1)])
def test_ms_read_vis_and_flags(orc, rows, nch, npol):
    rng = np.random.default_rng(rows * 100 + nch * 10 + npol)
    block = rng.standard_normal(rows * nch * npol * 2).astype(np.float32)
    vis = np.zeros(rows * nch, np.complex128)
    orc.orc_ms_read_vis(O.fp(block), rows, nch, npol, O.cp(vis))
    assert np.array_equal(vis, np_read_vis(block, rows, nch, npol))
    fl = (rng.random(rows * nch * npol) < 0.2).astype(np.uint8)
    out = np.zeros(rows * nch, np.uint8)
    n = orc.orc_ms_read_flag(O.bp(fl), rows, nch, npol, O.bp(out))
    f = fl.reshape(rows, nch, npol)
    ref = f[:, :, 0] != 0
    if npol == 4:
        ref = ref | (f[:, :, 3] != 0)
    assert np.array_equal(out, ref.T.reshape(-1).astype(np.uint8)) and n == int(ref.sum())


def test_ms_coords_sigma_and_write(orc):
    rng = np.random.default_rng(5)
    rows, nch = 333, 7
    uvw = rng.uniform(-4000, 4000, (rows, 3))
    uu, vv, ww = np.zeros(rows), np.zeros(rows), np.zeros(rows)
    lenv = orc.orc_ms_read_coords(O.dp(uvw.reshape(-1)), rows, O.dp(uu), O.dp(vv), O.dp(ww))
    assert np.array_equal(uu, uvw[:, 0]) and np.array_equal(vv, uvw[:, 1]) and np.array_equal(ww, uvw[:, 2])
    assert lenv == np.ceil(max(np.abs(uvw[:, 0]).max(), np.abs(uvw[:, 1]).max()))
    # SIGMA read flat: the first `rows` values squared, non-positive ones and the rest -> theory
    sig = rng.uniform(-1, 3, rows * 4).astype(np.float32)
    s2 = np.zeros(rows * nch, np.float32)
    orc.orc_ms_read_sigma2(O.fp(sig), rows, nch, np.float32(7.5), O.fp(s2))
    ref = np.full(rows * nch, np.float32(7.5))
    sq = sig[:rows] * sig[:rows]
    ref[:rows] = np.where(sq <= 0, np.float32(7.5), sq)
    assert np.array_equal(s2, ref)
    # write: [ch][row] uJy -> [row][ch] complex64 Jy
    vis = rng.standard_normal(rows * nch) + 1j * rng.standard_normal(rows * nch)
    out = np.zeros(rows * nch * 2, np.float32)
    orc.orc_ms_write_vis(O.cp(vis), rows, nch, O.fp(out))
    v = vis.reshape(nch, rows).T
    ref = np.stack([(v.real * 1e-6).astype(np.float32), (v.imag * 1e-6).astype(np.float32)], -1).reshape(-1)
    assert np.array_equal(out, ref)
