"""Channel sharding of the extraction across ranks (the reference's MPI decomposition).

The reference runs one rank per spectral window (RadioLensfit2.cpp:117-119): every rank grids
its own channels into facet partial sums (sum of visibilities, of variances, of weights), the
owner rank of a galaxy sums the partials of all ranks (data_processing-mpi.c:95-124), averages
them (average_facets, evaluate_uv_grid.c:216-230), fits, and broadcasts the result so that every
rank subtracts the fitted model from its own channels (data_processing-mpi.c:169-210).

Here that exchange is one all-reduce of the partial sums of a batch of galaxies (every rank then
holds the full facets and fits its share of the galaxies) and one all-gather of the fit results.
The collectives go through torch.distributed (NCCL between GPUs, gloo on CPU).  Galaxy fits are
independent, so galaxies are split across ranks round-robin like the reference's owner rule
(data_processing-mpi.c:71-93).
"""
from __future__ import annotations

import numpy as np

from . import constants as K


def channel_shards(n_ch: int, world: int):
    """Contiguous channel ranges [(lo, hi)] of each rank; sizes differ by at most one."""
    base, extra = divmod(n_ch, world)
    out, lo = [], 0
    for r in range(world):
        hi = lo + base + (1 if r < extra else 0)
        out.append((lo, hi))
        lo = hi
    return out


def owner_of(galaxy_index: int, world: int) -> int:
    """Round-robin owner rank of a galaxy (data_processing-mpi.c:71-93)."""
    return galaxy_index % world


def grid_partial_sums(uu, vv, wavenumbers, vis, sigma2, flag, length, facet, ch_lo, ch_hi):
    """Partial facet sums of channels [ch_lo, ch_hi) of a channel-major visibility array:
    (sum vis [F*F] complex, sum sigma2 [F*F], sum weights [F*F]) with the cell rule of
    evaluate_uv_grid.c:160-177 (uniform weights).  Host reference used by the shard tests."""
    n_rows = len(uu)
    nc = facet * facet
    inc = 2 * length / facet
    sv = np.zeros(nc, np.complex128)
    ss = np.zeros(nc)
    sw = np.zeros(nc)
    for ch in range(ch_lo, ch_hi):
        il = wavenumbers[ch] / (2.0 * np.pi)
        pu = ((uu * il + length) / inc).astype(np.int64)
        pv = ((vv * il + length) / inc).astype(np.int64)
        pc = pv * facet + pu
        sl = slice(ch * n_rows, (ch + 1) * n_rows)
        keep = (flag[sl] == 0) & (pc < nc)
        np.add.at(sv, pc[keep], vis[sl][keep])
        np.add.at(ss, pc[keep], sigma2[sl][keep].astype(np.float64))
        np.add.at(sw, pc[keep], 1.0)
    return sv, ss, sw


def average_facet(sv, ss, sw, length, facet):
    """average_facets + evaluate_facet_coords (evaluate_uv_grid.c:113-133, 216-230) of summed
    partials: compacted (u, v, vis/sigma2, sigma2) of the non-empty cells in row-major order."""
    nz = np.nonzero(sw)[0]
    inc = 2 * length / facet
    i, j = nz % facet, nz // facet
    gu = (i + 0.5) * inc - length
    gv = (j + 0.5) * inc - length
    vis = sv[nz] * sw[nz] / ss[nz]
    s2 = ss[nz] / (sw[nz] * sw[nz])
    return gu, gv, vis, s2


def allreduce_partials(sv, ss, sw, group=None):
    """Sum the partial facet arrays of all ranks (in place semantics, returns new arrays)."""
    import torch
    import torch.distributed as dist
    buf = torch.from_numpy(np.concatenate([sv.real, sv.imag, ss, sw]).astype(np.float64))
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    nc = len(ss)
    a = buf.numpy()
    return a[:nc] + 1j * a[nc:2 * nc], a[2 * nc:3 * nc].copy(), a[3 * nc:].copy()


def allgather_results(local: np.ndarray, n_total: int, world: int, rank: int, group=None) -> np.ndarray:
    """Every rank holds the fit results of its own galaxies (rows g with owner_of(g) == rank, the
    others zero); the sum over ranks is the complete table (the reference's MPI_Bcast of results,
    data_processing-mpi.c:169)."""
    import torch
    import torch.distributed as dist
    buf = torch.from_numpy(np.ascontiguousarray(local, dtype=np.float64))
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    return buf.numpy().copy()


# ------------------------------------------------------------------ shards on GPUs
def shard_observation(obs, world: int, rank: int):
    """The observation of rank `rank`: its contiguous channels, the full uvw, and the facet extent
    len of the whole observation (the reference exchanges len so that every rank grids on the same
    cells, RadioLensfit2.cpp:410-417)."""
    import dataclasses
    lo, hi = channel_shards(obs.n_ch, world)[rank]
    return dataclasses.replace(obs, wavenumbers=obs.wavenumbers[lo:hi].copy(), spec=obs.spec[lo:hi].copy(),
                               n_ch=hi - lo), (lo, hi)


class LocalExchange:
    """The exchange of simulated shards held by one process (one GPU): partial sums added in rank
    order (deterministic), results shared as they are."""

    def allreduce(self, parts):
        out = np.zeros_like(parts[0])
        for p in parts:
            out += p
        return out


class TorchExchange:
    """The exchange between ranks over torch.distributed: all-reduce of the partial facet sums of a
    round (NCCL between GPUs, gloo on CPU) and all-reduce of the owned results (the reference's
    MPI_Send/Recv of partials and MPI_Bcast of results, data_processing-mpi.c:95-169)."""

    def __init__(self, group=None, device=None):
        self.group, self.device = group, device

    def allreduce(self, arr):
        import torch
        import torch.distributed as dist
        t = torch.from_numpy(np.ascontiguousarray(arr, np.float64))
        if self.device is not None:
            t = t.to(self.device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=self.group)
        return t.cpu().numpy()


RESULT_FIELDS = ("e1", "e2", "var_e1", "var_e2", "oneDimvar", "maxL", "error", "iters", "nevals")


def fit_partials(partials, cat, length, fit_precision=0, gaussian=0):
    """rlf_fit_partials: the facets of summed partials fitted by the persistent fit kernel."""
    import ctypes as C
    from . import _lib
    from .pipeline import RESULT_DTYPE
    lib = _lib.load()
    P = np.ascontiguousarray(partials, np.float64)
    n, four, stride = P.shape
    ro = np.ascontiguousarray(K.ro_grid(), np.float64)
    opt = _lib.Options()
    opt.fit_precision, opt.gaussian = int(fit_precision), int(gaussian)
    out = (_lib.FitResult * n)()
    flux = np.ascontiguousarray(cat.flux, np.float64)
    scale = np.ascontiguousarray(cat.scale, np.float64)
    if lib.rlf_fit_partials(n, P.ctypes.data_as(_lib.PD), stride, flux.ctypes.data_as(_lib.PD),
                            scale.ctypes.data_as(_lib.PD), float(length), len(ro), ro.ctypes.data_as(_lib.PD),
                            C.byref(opt), out):
        raise RuntimeError("rlf_fit_partials failed")
    return np.frombuffer(out, dtype=RESULT_DTYPE, count=n).copy()


class ShardPipeline:
    """The path of data_processing-mpi.c on channel shards: galaxies in rounds of `round_size` in
    catalogue order; per round every shard extracts un-averaged facet partials over its channels
    (rlf_obs_facet_partials), the partials are summed across shards, the owner of each galaxy fits
    the summed facet (rlf_fit_partials; round-robin owners, data_processing-mpi.c:71-93), the
    results are shared, and every shard removes the good fits from its channels (rlf_obs_remove);
    then the re-fit pass over the bad galaxies, whose fits are removed when good and written with
    e = 0 when bad (data_processing.c:97-103).  With round_size 1 the order is the serial
    reference's; the reference's MPI run corresponds to round_size = number of ranks."""

    def __init__(self, devs, exchange, world=1, rank=0, fit_precision=0):
        self.devs = devs              # this process's shards (one per GPU rank, several when simulated)
        self.exchange = exchange
        self.world, self.rank = world, rank
        self.fit_precision = fit_precision

    def _round(self, cat, idx, stride):
        from .pipeline import RESULT_DTYPE
        sub = cat.subset(idx)
        parts = [d.facet_partials(sub, stride) for d in self.devs]
        local = parts[0] if len(parts) == 1 else LocalExchange().allreduce(parts)
        total = self.exchange.allreduce(local) if self.world > 1 else local
        own = np.array([owner_of(int(g), self.world) == self.rank for g in idx])
        res = np.zeros(len(idx), RESULT_DTYPE)
        if own.any():
            res[own] = fit_partials(total[own], sub.subset(np.nonzero(own)[0]), self.devs[0].obs.len_lambda,
                                    self.fit_precision)
        if self.world > 1:
            table = np.stack([res[f].astype(np.float64) for f in RESULT_FIELDS], 1)
            table = self.exchange.allreduce(np.where(own[:, None], table, 0.0))
            for k, f in enumerate(RESULT_FIELDS):
                res[f] = table[:, k].astype(res[f].dtype)
        for d in self.devs:
            d.remove(sub, res)
        return res

    def process(self, cat, round_size=1, refit=True):
        from .pipeline import RESULT_DTYPE
        stride = K.facet_size(K.RMAX, self.devs[0].obs.len_lambda) ** 2
        out = np.zeros(cat.n, RESULT_DTYPE)
        for a in range(0, cat.n, round_size):
            idx = np.arange(a, min(cat.n, a + round_size))
            out[idx] = self._round(cat, idx, stride)
        bad = np.nonzero(out["error"] != 0)[0]
        if refit and len(bad):
            for a in range(0, len(bad), round_size):
                idx = bad[a:a + round_size]
                r = self._round(cat, idx, stride)
                r["e1"] = np.where(r["error"] != 0, 0.0, r["e1"])
                r["e2"] = np.where(r["error"] != 0, 0.0, r["e2"])
                out[idx] = r
        return out
