"""Channel shards on one GPU (the reference's MPI decomposition, data_processing-mpi.c:65-216,
simulated as three observations of two channels each in one process): the shards' un-averaged
facet partials (rlf_obs_facet_partials) add up to the unsharded observation's partials (weights
exactly: integer counts; sums to 1e-13 relative, the summation grouping differs), and the shard
pipeline (partials summed across shards, facets fitted from the sums, fits removed from every
shard) with one galaxy per round reproduces the oracle's serial data_processing: error flags
equal, e within 1e-7, every shard's final data within 1e-11 of the oracle's channels."""
import numpy as np
import pytest

from radiolensfit2_gb300 import _lib, shard, constants as K
from radiolensfit2_gb300.pipeline import DeviceObservation

import _oracle as O
from _cases import Case, oracle_sky_model, oracle_data_processing

pytestmark = pytest.mark.gpu


def test_channel_shards_match_unsharded_and_oracle():
    orc = O.load_oracle()
    case = Case(n_ch=6, n_gal=6, flag_frac=0.03)
    o = case.obs
    sky = oracle_sky_model(orc, case)
    d_ref, s_ref, _, bl, ref = oracle_data_processing(orc, case, case.data, sky)
    nb = int(np.sum([r[6] for r in ref]))
    d_ref2, s_ref2, _, _, ref2 = oracle_data_processing(orc, case, d_ref, s_ref, re_fitting=True, bad_list=bl[:nb])
    world = 3
    devs = []
    for r in range(world):
        so, (lo, hi) = shard.shard_observation(o, world, r)
        sl = slice(lo * o.n_rows, hi * o.n_rows)
        d = DeviceObservation(so, precision=_lib.RLF_F64, sigma2=case.sigma2[sl], flag=case.flag[sl])
        d.set_vis(case.data[sl], sky[sl])
        devs.append((d, sl))
    full = DeviceObservation(o, precision=_lib.RLF_F64, sigma2=case.sigma2, flag=case.flag)
    full.set_vis(case.data, sky)
    stride = K.facet_size(K.RMAX, case.len) ** 2
    P = full.facet_partials(case.cat, stride)
    Ps = shard.LocalExchange().allreduce([d.facet_partials(case.cat, stride) for d, _ in devs])
    assert np.array_equal(P[:, 3], Ps[:, 3])
    assert np.array_equal(P[:, 2] != 0, Ps[:, 2] != 0)
    for a in range(3):
        assert np.max(np.abs(P[:, a] - Ps[:, a])) <= 1e-13 * np.max(np.abs(P[:, a]))
    full.close()
    pipe = shard.ShardPipeline([d for d, _ in devs], shard.LocalExchange())
    res = pipe.process(case.cat, round_size=1, refit=True)
    err_ref = np.array([r[6] for r in ref])
    for k, g in enumerate(bl[:nb]):  # the re-fit pass's results replace the bad ones
        err_ref[g] = ref2[k][6]
    e_ref = np.array([(r[0], r[1]) for r in ref])
    for k, g in enumerate(bl[:nb]):
        e_ref[g] = (ref2[k][0], ref2[k][1]) if ref2[k][6] == 0 else (0.0, 0.0)
    assert np.array_equal(res["error"], err_ref)
    assert np.max(np.abs(res["e1"] - e_ref[:, 0])) < 1e-7 and np.max(np.abs(res["e2"] - e_ref[:, 1])) < 1e-7
    for d, sl in devs:
        data, skym = d.get_vis()
        assert np.max(np.abs(data - d_ref2[sl])) < 1e-11 * np.max(np.abs(d_ref2))
        assert np.max(np.abs(skym - s_ref2[sl])) < 1e-11 * np.max(np.abs(sky))
        d.close()


def test_mixed_partials_batched():
    """FP32 observations extract the partials with the sequential batch extraction's first round
    (every galaxy against the same data): against the FP64 observation's partials of the same
    FP32-representable data (weights and variance sums equal, the sums within 2e-6 of their
    largest magnitude), and the sum of three 16-channel shards against the unsharded 48-channel
    observation (another chunking of the FP32 channel passes: the same bound)."""
    orc = O.load_oracle()
    case = Case(n_ant=40, ha_hours=2.0, dt_s=600.0, n_ch=48, n_gal=12, fmin=30.0, fmax=200.0, noise=1500.0,
                flag_frac=0.01)
    o = case.obs
    data = case.data.astype(np.complex64).astype(np.complex128)
    sky = oracle_sky_model(orc, case).astype(np.complex64).astype(np.complex128)
    stride = K.facet_size(K.RMAX, case.len) ** 2
    parts = {}
    for name, prec in (("f64", _lib.RLF_F64), ("mixed", _lib.RLF_MIXED)):
        d = DeviceObservation(o, precision=prec, sigma2=case.sigma2, flag=case.flag)
        d.set_vis(data, sky)
        parts[name] = d.facet_partials(case.cat, stride)
        d.close()
    shards = []
    for r in range(3):
        so, (lo, hi) = shard.shard_observation(o, 3, r)
        sl = slice(lo * o.n_rows, hi * o.n_rows)
        d = DeviceObservation(so, precision=_lib.RLF_MIXED, sigma2=case.sigma2[sl], flag=case.flag[sl])
        d.set_vis(data[sl], sky[sl])
        shards.append(d.facet_partials(case.cat, stride))
        d.close()
    parts["shards"] = shard.LocalExchange().allreduce(shards)
    ref = parts["f64"]
    for name in ("mixed", "shards"):
        P = parts[name]
        assert np.array_equal(P[:, 3], ref[:, 3]), name
        assert np.allclose(P[:, 2], ref[:, 2], rtol=1e-14, atol=0.0), name
        for a in range(2):
            err = np.max(np.abs(P[:, a] - ref[:, a]))
            print(f"{name} component {a}: max |d| {err:.3e} of {np.max(np.abs(ref[:, a])):.3e}")
            assert err <= 2e-6 * np.max(np.abs(ref[:, a])), name
