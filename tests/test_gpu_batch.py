"""Batch contexts (trans_batch_*) through the C ABI: cases added and removed while the context
runs give the same results as each case run alone.

Tolerance: bit-identical (0).  Every kernel computes a cell from its own case's data only, and
the sweep schedules compute every increment with the same operations, so the other cases of a
batch cannot change a case's arithmetic.
"""
import numpy as np
import pytest

from helpers import bit_equal_fraction, interior, small_cascade, small_channel

pytestmark = pytest.mark.gpu


def _case_a():
    return small_cascade(Kind_Spatial=3, Kind_Roe=3)


def _case_b():
    return small_channel(Kind_Spatial=2, Kind_Roe=1)


def _case_c():
    from trans_gb300 import case as CS
    from trans_gb300 import cases
    from helpers import SMALL_CASCADE
    c = cases.cascade(**dict(SMALL_CASCADE, nk=6), p_ratio=0.9, Kind_Spatial=3, Kind_Roe=3)
    conns, geo = CS.compute_geometry(c)
    st = CS.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    return c, conns, geo, st


def _fields(bt, cid, case):
    return [bt.get_field(cid, ib, "V") for ib in range(len(case.blocks))]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_case_alone_equals_case_in_mix(gpu_lib, precision):
    from trans_gb300 import abi
    from trans_gb300.solver import Batch
    prec = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
    a = _case_a()
    alone = Batch(prec)
    ia = alone.add(*a)
    alone.iterate(6)
    va = _fields(alone, ia, a[0])
    _, _, last_alone = alone.norms(ia)
    alone.close()

    mix = Batch(prec)
    ib = mix.add(*_case_b())
    mix.iterate(2)
    a2 = _case_a()
    ia2 = mix.add(*a2)
    mix.iterate(3)
    mix.remove(ib)
    ic = mix.add(*_case_c())
    mix.iterate(3)
    it, _, last_mix = mix.norms(ia2)
    assert it == 6
    vm = _fields(mix, ia2, a2[0])
    for q, b in enumerate(a[0].blocks):
        assert bit_equal_fraction(vm[q], va[q], interior(b.dims)) == 1.0, f"block {b.id}"
    for x, y in zip(last_mix, last_alone):
        assert x["DRSa"] == y["DRSa"]
    assert mix.norms(ic)[0] == 3
    mix.close()


def test_batch_matches_single_case_api(gpu_lib):
    """One case in a batch context and the same case through trans_create/trans_iterate."""
    from trans_gb300.solver import Batch, Solver
    c, conns, geo, st = _case_a()
    s = Solver(c, conns, geo, st)
    hist = [[n["DRSa"] for n in s.iterate(k)] for k in range(1, 6)]
    v_single = [s.get_field(q, "V") for q in range(len(c.blocks))]
    s.close()
    c, conns, geo, st = _case_a()
    bt = Batch()
    cid = bt.add(c, conns, geo, st)
    for k in range(5):
        bt.iterate(1)
        _, first, last = bt.norms(cid)
        assert [n["DRSa"] for n in last] == hist[k]
    assert [n["DRSa"] for n in first] == hist[0]
    for q, b in enumerate(c.blocks):
        assert bit_equal_fraction(bt.get_field(cid, q, "V"), v_single[q], interior(b.dims)) == 1.0
    bt.close()


def test_admission_by_device_budget(gpu_lib):
    from trans_gb300.solver import Batch
    a, b = _case_a(), _case_b()
    probe = Batch()
    need_a, need_b = probe.case_bytes(a[0], a[1]), probe.case_bytes(b[0], b[1])
    probe.close()
    assert need_a > 0 and need_b > 0
    bt = Batch(budget_bytes=need_a + need_b // 2)
    ia = bt.add(*a)
    assert ia is not None and bt.bytes_in_use() == need_a
    assert bt.add(*b) is None                     # does not fit: refused, nothing allocated
    assert bt.bytes_in_use() == need_a
    bt.iterate(2)
    bt.remove(ia)
    assert bt.bytes_in_use() == 0
    ib = bt.add(*_case_b())
    assert ib is not None
    bt.iterate(1)
    assert bt.norms(ib)[0] == 1
    assert np.isfinite(bt.norms(ib)[2][0]["DRSa"])
    bt.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_equals_direct_launches(gpu_lib, precision, monkeypatch):
    """Whole iterations replayed as one CUDA graph give the same state as launching every
    kernel directly (TRANS_GRAPHS=0)."""
    from trans_gb300 import abi
    from trans_gb300.solver import Batch
    prec = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
    out = {}
    for graphs in ("1", "0"):
        monkeypatch.setenv("TRANS_GRAPHS", graphs)
        c, conns, geo, st = _case_a()
        bt = Batch(prec)
        cid = bt.add(c, conns, geo, st)
        bt.iterate(9)
        out[graphs] = (_fields(bt, cid, c), bt.norms(cid))
        bt.close()
    for q, b in enumerate(c.blocks):
        assert bit_equal_fraction(out["1"][0][q], out["0"][0][q], interior(b.dims)) == 1.0
    assert out["1"][1][0] == out["0"][1][0] == 9
    assert [n["DRSa"] for n in out["1"][1][2]] == [n["DRSa"] for n in out["0"][1][2]]
