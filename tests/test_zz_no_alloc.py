"""rlf_gridding_visibilities_noalloc against the allocating drop-in gridding_visibilities.

The no-allocation entry point exists for callers that cannot allocate device memory, such as
code inside a framework that owns the device heap (a caching allocator or a fixed pool) or a
real-time caller that forbids allocation after start-up.  Such a caller passes its own device
buffers, and the library grids with a fixed scratch array of its own device memory.  The test
allocates the device buffers itself (with torch) and compares three calls in a row with the
host-pointer entry point: a large facet, a small one, and the large one again, so that partial
sums the previous call left in the shared scratch cannot leak into a result.

This file is named to be collected last, so that a run which stops at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from radiolensfit2_gb300 import _lib
from radiolensfit2_gb300.abi import bptr, cptr, dptr, fptr

import _oracle as O
from _cases import Case

pytestmark = pytest.mark.gpu


def _oracle_grid(wn, n_ch, u, v, vis, s2, flag, length, F):
    orc = O.load_oracle()
    nc = F * F
    gv, gs, sw = np.zeros(nc, np.complex128), np.zeros(nc), np.zeros(nc)
    orc.orc_gridding(O.dp(wn), n_ch, len(u), O.dp(u), O.dp(v), O.cp(vis), O.fp(s2), length, F, O.cp(gv), O.dp(gs),
                     O.bp(flag), O.dp(sw))
    return gv, gs, sw


def _noalloc(lib, torch, dev, wn, n_ch, d_u, d_v, d_vis, d_s2, d_flag, n_rows, length, F):
    nc = F * F
    out_vis = torch.full((2 * nc,), float("nan"), dtype=torch.float64, device=dev)
    out_s2 = torch.full((nc,), float("nan"), dtype=torch.float64, device=dev)
    out_sw = torch.full((nc,), float("nan"), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    rc = lib.rlf_gridding_visibilities_noalloc(
        dptr(wn), n_ch, n_rows, d_u.data_ptr(), d_v.data_ptr(), d_vis.data_ptr(), d_s2.data_ptr(),
        d_flag.data_ptr(), length, F, out_vis.data_ptr(), out_s2.data_ptr(), out_sw.data_ptr(), None)
    assert rc == 0
    return out_vis.cpu().numpy().view(np.complex128), out_s2.cpu().numpy(), out_sw.cpu().numpy()


def _reference(lib, case, F):
    o = case.obs
    nc = F * F
    vis, s2, sw = np.zeros(nc, np.complex128), np.zeros(nc), np.zeros(nc)
    lib.gridding_visibilities(dptr(o.wavenumbers), o.n_ch, o.n_rows, dptr(o.uu), dptr(o.vv), cptr(case.data),
                              fptr(case.sigma2), case.len, F, cptr(vis), dptr(s2), bptr(case.flag), dptr(sw))
    return vis, s2, sw


def test_noalloc_gridding_matches_gridding_visibilities():
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    case = Case(flag_frac=0.03)
    o = case.obs
    dev = torch.device("cuda", 0)

    def on_device(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    d_u, d_v = on_device(o.uu), on_device(o.vv)
    d_vis = on_device(case.data.view(np.float64))      # complex128 as (re, im) pairs
    d_s2 = on_device(case.sigma2)
    d_flag = on_device(case.flag.view(np.uint8))
    torch.cuda.synchronize()
    for F in (34, 10, 34, 40, 48):
        nc = F * F
        out_vis = torch.full((2 * nc,), float("nan"), dtype=torch.float64, device=dev)
        out_s2 = torch.full((nc,), float("nan"), dtype=torch.float64, device=dev)
        out_sw = torch.full((nc,), float("nan"), dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = lib.rlf_gridding_visibilities_noalloc(
            dptr(o.wavenumbers), o.n_ch, o.n_rows, d_u.data_ptr(), d_v.data_ptr(), d_vis.data_ptr(),
            d_s2.data_ptr(), d_flag.data_ptr(), case.len, F, out_vis.data_ptr(), out_s2.data_ptr(),
            out_sw.data_ptr(), None)
        assert rc == 0
        vis_ref, s2_ref, sw_ref = _reference(lib, case, F)
        sw = out_sw.cpu().numpy()
        assert np.array_equal(sw, sw_ref)                 # cell counts: integer work, exact
        n = int(np.count_nonzero(sw_ref))
        vis = out_vis.cpu().numpy().view(np.complex128)[:n]
        s2 = out_s2.cpu().numpy()[:n]
        # the tolerances of the drop-in gridding test (summation order differs)
        assert np.max(np.abs(vis - vis_ref[:n])) < 1e-12 * np.max(np.abs(vis_ref[:n]))
        assert np.max(np.abs(s2 - s2_ref[:n])) < 1e-13 * np.max(np.abs(s2_ref[:n]))
        # and the oracle (the reference's gridding restated on the CPU)
        gv, gs, gw = _oracle_grid(o.wavenumbers, o.n_ch, o.uu, o.vv, case.data, case.sigma2, case.flag, case.len, F)
        assert np.array_equal(sw, gw)
        assert np.max(np.abs(vis - gv[:n])) < 1e-12 * np.max(np.abs(gv[:n]))
        assert np.max(np.abs(s2 - gs[:n])) < 1e-13 * np.max(np.abs(gs[:n]))
    # sizes beyond the scratch array are rejected before any launch
    big = torch.zeros(2 * 49 * 49, dtype=torch.float64, device=dev)
    rc = lib.rlf_gridding_visibilities_noalloc(
        dptr(o.wavenumbers), o.n_ch, o.n_rows, d_u.data_ptr(), d_v.data_ptr(), d_vis.data_ptr(),
        d_s2.data_ptr(), d_flag.data_ptr(), case.len, 49, big.data_ptr(), big.data_ptr(), big.data_ptr(), None)
    assert rc != 0


def test_noalloc_gridding_capped_blocks_largest_facet():
    """More rows than the scratch array's 64 partial facets cover at 2048 rows each (the grid is
    capped at 64 blocks, each taking several row ranges) at the largest accepted facet (48), whose
    reduced sums fill the end of the scratch array; against the oracle and the drop-in."""
    torch = pytest.importorskip("torch")
    lib = _lib.load()
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(11)
    n_rows, n_ch, length = 64 * 2048 + 9001, 2, 2.4e4
    wn = np.array([2 * np.pi * 950.12e6 / 299792458.0, 2 * np.pi * 950.36e6 / 299792458.0])
    lam = 2 * np.pi / wn[-1]
    u = rng.uniform(-0.97, 0.97, n_rows) * length * lam
    v = rng.uniform(-0.97, 0.97, n_rows) * length * lam
    vis = (rng.standard_normal(n_ch * n_rows) + 1j * rng.standard_normal(n_ch * n_rows)) * 7.5e4
    s2 = np.full(n_ch * n_rows, np.float32(5.6e9), np.float32)
    flag = (rng.random(n_ch * n_rows) < 0.02).astype(np.uint8)
    on = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_u, d_v, d_vis, d_s2, d_flag = on(u), on(v), on(vis.view(np.float64)), on(s2), on(flag)
    for F in (48, 48):  # two calls in a row: the second must not see the first's sums
        gvis, gs2, gsw = _noalloc(lib, torch, dev, wn, n_ch, d_u, d_v, d_vis, d_s2, d_flag, n_rows, length, F)
        ov, os2, osw = _oracle_grid(wn, n_ch, u, v, vis, s2, flag, length, F)
        assert np.array_equal(gsw, osw)
        n = int(np.count_nonzero(osw))
        assert n > 2000
        assert np.max(np.abs(gvis[:n] - ov[:n])) < 1e-12 * np.max(np.abs(ov[:n]))
        assert np.max(np.abs(gs2[:n] - os2[:n])) < 1e-13 * np.max(np.abs(os2[:n]))
        nc = F * F
        dv, ds2, dsw = np.zeros(nc, np.complex128), np.zeros(nc), np.zeros(nc)
        lib.gridding_visibilities(dptr(wn), n_ch, n_rows, dptr(u), dptr(v), cptr(vis), fptr(s2), length, F,
                                  cptr(dv), dptr(ds2), bptr(flag), dptr(dsw))
        assert np.array_equal(gsw, dsw)
        assert np.max(np.abs(gvis[:n] - dv[:n])) < 1e-12 * np.max(np.abs(dv[:n]))
