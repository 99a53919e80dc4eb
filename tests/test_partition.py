"""Block decomposition of one case over ranks (trans_gb300.partition): the cross-rank 1-to-1
interface exchange of BC/PARALLEL_BC_P2P.F90, run as gloo ranks on the CPU with the oracle as
each rank's solver.  The five-block cascade split over two ranks must reproduce the
single-process run bit for bit: the halos carry exactly what the same-rank interface copy
reads, and every other stage is block-local."""
import os
import socket

import numpy as np
import pytest

from helpers import SMALL_CASCADE, interior

ITERS = 8


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case(**sw):
    from trans_gb300 import case as CS
    from trans_gb300 import cases
    c = cases.cascade(**SMALL_CASCADE, **sw)
    conns, geo = CS.compute_geometry(c)
    st = CS.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    return c, conns, geo, st


def _rank(rank, world, port, sw, out):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch.distributed as dist
    from oracle.oracle import OracleSolver, load
    from trans_gb300 import partition as P
    try:
        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
        load().oracle_set_threads(1)
        c, conns, geo, st = _case(**sw)
        owner = P.partition_blocks(c.blocks, world)
        mine = P.local_case(c, owner, rank)
        segs = P.halo_segments(c, conns, owner, rank)
        s = OracleSolver(mine, conns, geo, st)
        drv = P.StageDriver(s, P.HaloExchange(s.lib, "oracle_", s.ctx, segs, P.torch_transport()))
        hist = [[n["DRSa"] for n in drv.iterate(ki)] for ki in range(1, ITERS + 1)]
        fields = {b.id: {f: s.get_field(ib, f) for f in ("V", "PP", "T", "RMIU")} for ib, b in enumerate(mine.blocks)}
        out.put((rank, [b.id for b in mine.blocks], len(segs), drv.x.words_moved, hist, fields, None))
        s.close()
        dist.barrier()
        dist.destroy_process_group()
    except Exception as e:          # reported to the parent, which fails the test
        import traceback
        out.put((rank, None, 0, 0, None, None, traceback.format_exc()))


def test_partition_balances_and_covers():
    from trans_gb300 import cases, partition as P
    c = cases.cascade(**cases.CASCADE_CONFIG2)
    owner = P.partition_blocks(c.blocks, 2)
    assert sorted(owner) == [b.id for b in c.blocks]
    load = [sum(int(np.prod([d - 1 for d in b.dims])) for b in c.blocks if owner[b.id] == r) for r in range(2)]
    assert sum(load) == 1966080
    assert min(load) >= 0.4 * sum(load)          # O-block alone (786,432) against the four others
    assert P.partition_blocks(c.blocks, 1) == {b.id: 0 for b in c.blocks}


@pytest.mark.parametrize("sw", [dict(Kind_Spatial=3, Kind_Roe=3), dict(Kind_Spatial=2, Kind_Roe=1)],
                         ids=["mdcd_ausmpw", "muscl_roe"])
def test_two_rank_split_matches_single_process(sw):
    torch = pytest.importorskip("torch")
    from oracle.oracle import OracleSolver, load
    from trans_gb300 import partition as P
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, sw, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=300) for _ in procs), key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
    for r in res:
        assert r[6] is None, r[6]
    for p in procs:
        assert p.exitcode == 0
    # the single-process oracle on the whole case
    load().oracle_set_threads(1)
    c, conns, geo, st = _case(**sw)
    ref = OracleSolver(c, conns, geo, st)
    href = [[n["DRSa"] for n in ref.iterate(ki)] for ki in range(1, ITERS + 1)]
    owner = P.partition_blocks(c.blocks, 2)
    assert sorted(res[0][1] + res[1][1]) == sorted(b.id for b in c.blocks)
    assert res[0][2] > 0 and res[1][2] > 0 and res[0][3] > 0          # both ranks exchanged halos
    for ib, b in enumerate(c.blocks):
        r = res[owner[b.id]]
        k = r[1].index(b.id)
        assert [h[k] for h in r[4]] == [h[ib] for h in href], f"block {b.id}: residual history differs"
        m = interior(b.dims)
        for f in ("V", "PP", "T", "RMIU"):
            a, e = r[5][b.id][f], ref.get_field(ib, f)
            assert np.array_equal(a[..., m].view(np.int64), e[..., m].view(np.int64)), f"block {b.id} {f} differs"
    ref.close()
