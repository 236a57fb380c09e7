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
