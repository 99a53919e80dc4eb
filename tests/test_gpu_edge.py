"""Edge cases through the C ABI: the smallest block the boundary tables accept (three interior
cells per direction, so every stencil reaches into ghosts on both sides at once), an empty batch
context, and a batch emptied by removals.  Tolerance: bit-identical to the oracle for the
FP64 state; the empty contexts answer with status codes and do no device work."""
import numpy as np
import pytest

from helpers import bit_equal_fraction, interior, small_channel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scheme", [dict(Kind_Spatial=3, Kind_Roe=3), dict(Kind_Spatial=2, Kind_Roe=1)],
                         ids=["mdcd_ausmpw", "muscl_roe"])
def test_smallest_block_bitwise(gpu_lib, scheme):
    from oracle.oracle import OracleSolver
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_channel(ni=4, nj=4, nk=4, **scheme)
    assert c.blocks[0].dims == (4, 4, 4)
    g = Solver(c, conns, geo, st, lib=gpu_lib)
    o = OracleSolver(c, conns, geo, st)
    for ki in range(1, 11):
        ng, no = g.iterate(ki), o.iterate(ki)
        assert abs(ng[0]["DRSa"] - no[0]["DRSa"]) <= 1e-11 * no[0]["DRSa"]
    m = interior(c.blocks[0].dims)
    for name in ("V", "PP", "T", "RMIU"):
        assert bit_equal_fraction(g.get_field(0, name), o.get_field(0, name), m) == 1.0, name
    g.close()


def test_smallest_block_mixed_runs(gpu_lib):
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_channel(ni=4, nj=4, nk=4, Kind_Spatial=3, Kind_Roe=3)
    c.params.precision = abi.TRANS_MIXED
    s = Solver(c, conns, geo, st, lib=gpu_lib)
    h = [s.iterate(ki)[0]["DRSa"] for ki in range(1, 11)]
    assert np.all(np.isfinite(h))
    s.close()


def test_empty_and_emptied_batch(gpu_lib):
    from trans_gb300 import abi
    from trans_gb300.solver import Batch
    bt = Batch(abi.TRANS_FP64, lib=gpu_lib)
    assert bt.iterate(3) is False                 # nothing to do: TRANS_OK
    assert bt.integrals() == {}
    assert bt.bytes_in_use() == 0
    cid = bt.add(*small_channel())
    assert bt.iterate(2) is False
    assert bt.norms(cid)[0] == 2
    bt.remove(cid)
    assert bt.bytes_in_use() == 0
    assert bt.iterate(1) is False
    assert gpu_lib.trans_batch_cases(bt.ctx, None, 0) == 0
    bt.close()
