"""Integrated quantities on the device (trans_get_integrals, trans_get_wall_cp and the batch
forms) against the host sums of trans_gb300.integrals over the same state.

Tolerances: the device sums the same per-face expressions in another order (a fixed-stride
split over 256 threads, then a tree), so mass flow, mass-averaged p0 and p agree to 1e-12
relative and the wall forces to 1e-12 of the largest component.  The pressure coefficient is
one expression per face: bit-identical.  The same state gives the same bits from every call,
and a case's sums do not depend on the other cases of a batch.
"""
import numpy as np
import pytest

from helpers import small_cascade, small_channel

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _host(c, conns, geo, fields):
    from trans_gb300 import integrals
    return integrals.face_integrals(c, conns, geo, fields)


def _close(dev, host):
    for k in ("mass_in", "p0_in", "p_in", "mass_out", "p0_out", "p_out"):
        assert abs(dev[k] - host[k]) <= TOL * abs(host[k]), k
    assert abs(dev["loss"] - host["loss"]) <= 1e-9 * max(abs(host["loss"]), 1e-3)
    for k in ("force_p", "force_v"):
        scale = max(abs(x) for x in host[k])
        assert scale > 0, k
        assert max(abs(x - y) for x, y in zip(dev[k], host[k])) <= TOL * scale, k


def _solver_fields(s, c):
    return [{f: s.get_field(ib, f) for f in ("V", "PP", "T")} for ib in range(len(c.blocks))]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("which", ["channel", "cascade"])
def test_device_integrals_match_host(gpu_lib, precision, which):
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_channel() if which == "channel" else small_cascade(Kind_Spatial=3, Kind_Roe=3)
    c.params.precision = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
    s = Solver(c, conns, geo, st, lib=gpu_lib)
    for ki in range(1, 5):
        s.iterate(ki)
    dev = s.integrals()
    host = _host(c, conns, geo, _solver_fields(s, c))
    _close(dev, host)
    assert dev["mass_in"] > 0 and dev["mass_out"] > 0
    again = s.integrals()
    assert again == dev                     # same state, same bits
    s.close()


def test_device_integrals_of_the_oracle_state(gpu_lib):
    """The FP64 library and the oracle advance the same state bit for bit, so the device sums
    of the library's state equal the host sums of the oracle's state."""
    from oracle.oracle import OracleSolver
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_channel()
    o = OracleSolver(c, conns, geo, st)
    s = Solver(c, conns, geo, st, lib=gpu_lib)
    for ki in range(1, 4):
        o.iterate(ki)
        s.iterate(ki)
    of = [{f: o.get_field(ib, f) for f in ("V", "PP", "T")} for ib in range(len(c.blocks))]
    _close(s.integrals(), _host(c, conns, geo, of))
    s.close()


def test_wall_cp_bit_identical(gpu_lib):
    from trans_gb300 import integrals
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    s = Solver(c, conns, geo, st, lib=gpu_lib)
    for ki in range(1, 4):
        s.iterate(ki)
    f = _solver_fields(s, c)
    n = 0
    for ib, b in enumerate(c.blocks):
        for ic, cn in enumerate(conns[b.id], start=1):
            if cn.BCType != 1:
                continue
            dev = s.wall_cp(ib, ic)
            host = integrals.segment_cp(c, conns, f, ib, ic)
            assert dev.shape == host.shape
            assert np.array_equal(dev.view(np.int64), host.view(np.int64)), (ib, ic)
            n += 1
    assert n >= 10
    from trans_gb300.solver import SolverError
    with pytest.raises(SolverError):
        s.wall_cp(0, 1)                     # a 1-to-1 interface, not a wall
    s.close()


def test_batch_integrals_alone_equal_in_mix(gpu_lib):
    from trans_gb300 import abi
    from trans_gb300.solver import Batch
    alone = Batch(abi.TRANS_FP64)
    ia = alone.add(*small_cascade(Kind_Spatial=3, Kind_Roe=3))
    alone.iterate(4)
    ref = alone.integrals(ia)
    alone.close()

    mix = Batch(abi.TRANS_FP64)
    ib = mix.add(*small_channel())
    a = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    ia2 = mix.add(*a)
    mix.iterate(4)
    every = mix.integrals()
    assert set(every) == {ib, ia2}
    assert every[ia2] == ref
    assert mix.integrals(ia2) == ref
    assert every[ib] == mix.integrals(ib)
    mix.remove(ib)
    assert mix.integrals(ia2) == ref         # rebuilt tables, same sums
    cp = mix.wall_cp(ia2, 0, 3)
    host_fields = [{f: mix.get_field(ia2, q, f) for f in ("V", "PP", "T")} for q in range(len(a[0].blocks))]
    from trans_gb300 import integrals
    assert np.array_equal(cp, integrals.segment_cp(a[0], a[1], host_fields, 0, 3))
    mix.close()


def test_wall_forces_per_face_and_moments(gpu_lib):
    """trans_get_wall_forces: the pressure and viscous force of every face of every wall
    segment, against the host restatement of the same per-face terms (the same expressions in
    FP64: 1e-12 of the segment's largest component; in practice bit-identical); summed over the
    walls they give trans_get_integrals' wall forces; and the moment sums of
    Output/OUTPUT_ClCdCm.F90:250-252 formed from them with the face centres equal the host
    moment sums."""
    from trans_gb300 import integrals
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    s = Solver(c, conns, geo, st, lib=gpu_lib)
    for ki in range(1, 4):
        s.iterate(ki)
    f = _solver_fields(s, c)
    dev_f, host_f, centres = [], [], []
    for ib, b in enumerate(c.blocks):
        for ic, cn in enumerate(conns[b.id], start=1):
            if cn.BCType != 1:
                continue
            dev = s.wall_forces(ib, ic)
            host = integrals.segment_wall_forces(c, conns, geo, f, ib, ic)
            assert dev.shape == host.shape
            scale = np.max(np.abs(host))
            assert np.max(np.abs(dev - host)) <= TOL * scale, (ib, ic)
            dev_f.append(dev)
            host_f.append(host)
            centres.append(integrals.segment_face_centres(c, conns, ib, ic))
    total = sum(F.sum(axis=1) for F in dev_f)
    intg = s.integrals()
    for q in range(3):
        assert abs(total[q] - intg["force_p"][q]) <= TOL * max(abs(x) for x in intg["force_p"])
        assert abs(total[3 + q] - intg["force_v"][q]) <= TOL * max(abs(x) for x in intg["force_v"])
    ref = (0.25, -0.1, 0.5)
    m_dev = integrals.wall_moments(dev_f, centres, ref)
    m_host = integrals.wall_moments(host_f, centres, ref)
    mscale = max(abs(x) for x in m_host)
    assert mscale > 0
    assert max(abs(a - b) for a, b in zip(m_dev, m_host)) <= TOL * mscale
    s.close()
