"""Multi-rank path on CPU (gloo, world size 2): channel shards grid their own channels, the
partial facet sums are all-reduced, the averaged facets equal the unsharded gridding of the
oracle; fit results are all-gathered."""
import os
import socket

import numpy as np
import pytest

from radiolensfit2_gb300 import shard, constants as K


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from _cases import Case
    case = Case(n_ch=6, flag_frac=0.05)
    o = case.obs
    F = 10
    lo, hi = shard.channel_shards(o.n_ch, world)[rank]
    sv, ss, sw = shard.grid_partial_sums(o.uu, o.vv, o.wavenumbers, case.data, case.sigma2, case.flag,
                                         case.len, F, lo, hi)
    sv, ss, sw = shard.allreduce_partials(sv, ss, sw)
    gu, gv, vis, s2 = shard.average_facet(sv, ss, sw, case.len, F)
    # fit results: each rank owns every world-th galaxy
    n = 7
    local = np.zeros((n, 3))
    for g in range(n):
        if shard.owner_of(g, world) == rank:
            local[g] = (g, 10.0 * g, rank)
    table = shard.allgather_results(local, n, world, rank)
    q.put((rank, gu, gv, vis, s2, sw, table))
    dist.destroy_process_group()


def test_channel_shards_partition():
    for n_ch in (1, 4, 7, 64):
        for world in (1, 2, 3, 8):
            s = shard.channel_shards(n_ch, world)
            assert s[0][0] == 0 and s[-1][1] == n_ch
            assert all(a[1] == b[0] for a, b in zip(s, s[1:]))
            sizes = [b - a for a, b in s]
            assert max(sizes) - min(sizes) <= 1


def test_two_rank_facet_reduction_matches_unsharded():
    import torch.multiprocessing as mp
    import _oracle as O
    from _cases import Case
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    case = Case(n_ch=6, flag_frac=0.05)
    o = case.obs
    F = 10
    orc = O.load_oracle()
    nc = F * F
    gv2, gs2, sw2 = np.zeros(nc, np.complex128), np.zeros(nc), np.zeros(nc)
    orc.orc_gridding(O.dp(o.wavenumbers), o.n_ch, o.n_rows, O.dp(o.uu), O.dp(o.vv), O.cp(case.data),
                     O.fp(case.sigma2), case.len, F, O.cp(gv2), O.dp(gs2), O.bp(case.flag), O.dp(sw2))
    n = int(np.count_nonzero(sw2))
    u2, v2 = np.zeros(nc), np.zeros(nc)
    orc.orc_facet_coords(O.dp(u2), O.dp(v2), case.len, F, O.dp(sw2))
    for rank, gu, gv, vis, s2, sw, table in got:
        assert np.array_equal(sw, sw2)                     # weights: integer sums, exact
        assert np.array_equal(gu, u2[:n]) and np.array_equal(gv, v2[:n])
        assert np.max(np.abs(vis - gv2[:n])) <= 1e-12 * np.max(np.abs(gv2[:n]))
        assert np.allclose(s2, gs2[:n], rtol=1e-14)
        assert table[:, 0].tolist() == list(range(7)) and table[:, 2].tolist() == [g % 2 for g in range(7)]
