"""Checkpoint and resume through restart files in the reference's layout: fields read back from
the GPU, written with trans_gb300.restart, and a resumed solve on the GPU bit-identical to the
oracle resumed from the same files."""
import pytest

from helpers import bit_equal_fraction, interior, small_cascade

pytestmark = pytest.mark.gpu


def test_gpu_checkpoint_resume_bitwise(gpu_lib, tmp_path):
    from oracle.oracle import OracleSolver
    from trans_gb300 import restart
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    g = Solver(c, conns, geo, st)
    for ki in range(1, 5):
        g.iterate(ki)
    fields = [{n: g.get_field(ib, n) for n in ("V", "RMIU", "WT0", "WT1")} for ib in range(len(c.blocks))]
    g.close()
    restart.save_case(str(tmp_path / "ck"), c, fields, ki=5)
    ki0, st2 = restart.restart_state(str(tmp_path / "ck"), c, geo)
    g = Solver(c, conns, geo, st2)
    o = OracleSolver(c, conns, geo, st2)
    for ki in range(ki0, ki0 + 4):
        g.iterate(ki)
        o.iterate(ki)
    for ib, b in enumerate(c.blocks):
        m = interior(b.dims)
        for n in ("V", "PP", "T", "RMIU"):
            frac = bit_equal_fraction(g.get_field(ib, n), o.get_field(ib, n), m)
            assert frac == 1.0, (b.id, n, frac)
    g.close()
    o.close()
