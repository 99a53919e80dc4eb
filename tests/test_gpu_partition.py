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
