"""The block decomposition of one case on the device: the five-block cascade split over two
contexts (two ranks' shares of the blocks), whose cross-rank 1-to-1 interfaces are exchanged
with trans_halo_pack / trans_halo_unpack after the state and gradient ghost passes (the
reference's PARALLEL_BCs, BC/PARALLEL_BC_P2P.F90), iterates exactly as the whole case in one
context.  Both shares run on the one GPU in lockstep, stage by stage, with the buffers handed
over on the host; no kernel waits on another context.  Bar: FP64 states and residual
histories bit-identical; the mixed path (residual form fixed so both runs sum alike) as well.
"""
import numpy as np
import pytest

from helpers import SMALL_CASCADE, bit_equal_fraction, interior

pytestmark = pytest.mark.gpu

ITERS = 6


def _case(precision, **sw):
    from trans_gb300 import abi
    from trans_gb300 import case as CS
    from trans_gb300 import cases
    c = cases.cascade(**SMALL_CASCADE, **sw)
    c.params.precision = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
    conns, geo = CS.compute_geometry(c)
    st = CS.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    return c, conns, geo, st


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("sw", [dict(Kind_Spatial=3, Kind_Roe=3), dict(Kind_Spatial=2, Kind_Roe=1)],
                         ids=["mdcd_ausmpw", "muscl_roe"])
def test_two_context_split_matches_whole_case(gpu_lib, monkeypatch, precision, sw):
    from trans_gb300 import partition as P
    from trans_gb300.solver import Solver
    monkeypatch.setenv("TRANS_RESID_TMA", "0")
    c, conns, geo, st = _case(precision, **sw)
    owner = P.partition_blocks(c.blocks, 2)
    ranks = []
    for r in range(2):
        mine = P.local_case(c, owner, r)
        segs = P.halo_segments(c, conns, owner, r)
        assert segs, "every share has cross-rank interfaces"
        s = Solver(mine, conns, geo, st, lib=gpu_lib)
        ranks.append((mine, s, P.HaloExchange(s.lib, "trans_", s.ctx, segs, None)))
    whole = Solver(c, conns, geo, st, lib=gpu_lib)
    hist_split = {b.id: [] for b in c.blocks}
    hist_whole = {b.id: [] for b in c.blocks}
    for ki in range(1, ITERS + 1):
        for stage in P.STAGES:
            for mine, s, x in ranks:
                s.run_stage(stage, ki)
            if stage in ("BC_STATE", "BC_GRAD"):
                sweep = -1 if stage == "BC_STATE" else 0
                mail, packed = {}, []
                for mine, s, x in ranks:
                    sends, recvs = x.pack_all(sweep)
                    for peer, key, buf in sends:
                        mail[key] = buf
                    packed.append(recvs)
                for (mine, s, x), recvs in zip(ranks, packed):
                    x.unpack_all(sweep, {key: mail[key] for peer, key, words in recvs})
        for mine, s, x in ranks:
            s.run_stage("UPDATE_U", ki)
            for b, n in zip(mine.blocks, s.norms()):
                hist_split[b.id].append(n["DRSa"])
        for b, n in zip(c.blocks, whole.iterate(ki)):
            hist_whole[b.id].append(n["DRSa"])
    for b in c.blocks:
        assert hist_split[b.id] == hist_whole[b.id], f"block {b.id}: residual history differs"
    for ib, b in enumerate(c.blocks):
        r = owner[b.id]
        mine, s, x = ranks[r]
        jb = [q.id for q in mine.blocks].index(b.id)
        m = interior(b.dims)
        for name in ("V", "PP", "T", "RMIU"):
            frac = bit_equal_fraction(s.get_field(jb, name), whole.get_field(ib, name), m)
            assert frac == 1.0, f"block {b.id} {name}: {frac:.6f} bit-identical"
    assert all(x.words_moved > 0 for _, _, x in ranks)
    for _, s, _ in ranks:
        s.close()
    whole.close()


def _rank(rank, world, port, out):
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    try:
        import torch.distributed as dist
        from trans_gb300 import partition as P
        from trans_gb300.solver import Solver
        dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
        c, conns, geo, st = _case("fp64", Kind_Spatial=3, Kind_Roe=3)
        owner = P.partition_blocks(c.blocks, world)
        mine = P.local_case(c, owner, rank)
        s = Solver(mine, conns, geo, st)
        drv = P.StageDriver(s, P.HaloExchange(s.lib, "trans_", s.ctx, P.halo_segments(c, conns, owner, rank),
                                              P.torch_transport()))
        hist = [[n["DRSa"] for n in drv.iterate(ki)] for ki in range(1, ITERS + 1)]
        fields = {b.id: {f: s.get_field(ib, f) for f in ("V", "PP")} for ib, b in enumerate(mine.blocks)}
        out.put((rank, [b.id for b in mine.blocks], hist, fields, None))
        s.close()
        dist.barrier()
        dist.destroy_process_group()
    except Exception:                       # reported to the parent, which fails the test
        import traceback
        out.put((rank, None, None, None, traceback.format_exc()))


def test_two_process_split_with_torch_transport(gpu_lib):
    """The same split as two processes (two ranks on the one GPU, each its own CUDA context),
    the segments moved by torch.distributed point-to-point operations over gloo
    (partition.torch_transport) and each rank driven by partition.StageDriver: every block's
    state and residual history bit-identical to the whole case in one context."""
    import socket
    import torch
    from trans_gb300 import partition as P
    from trans_gb300.solver import Solver
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    procs = [mp.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted((q.get(timeout=600) for _ in procs), key=lambda x: x[0])
    for p in procs:
        p.join(timeout=120)
    for r in res:
        assert r[4] is None, r[4]
    c, conns, geo, st = _case("fp64", Kind_Spatial=3, Kind_Roe=3)
    whole = Solver(c, conns, geo, st, lib=gpu_lib)
    href = [[n["DRSa"] for n in whole.iterate(ki)] for ki in range(1, ITERS + 1)]
    owner = P.partition_blocks(c.blocks, 2)
    for ib, b in enumerate(c.blocks):
        r = res[owner[b.id]]
        k = r[1].index(b.id)
        assert [h[k] for h in r[2]] == [h[ib] for h in href], f"block {b.id}: residual history differs"
        m = interior(b.dims)
        for f in ("V", "PP"):
            assert bit_equal_fraction(r[3][b.id][f], whole.get_field(ib, f), m) == 1.0, (b.id, f)
    whole.close()
