"""Bounded device-side waits: a cooperative LU-SGS sweep schedule whose waits are allowed no
polls at all (TRANS_SWEEP_SPIN=0) gives up, records the error and returns; the host reports
TRANS_E_TIMEOUT from the UPDATE stage and from trans_update_static_scratch, and the CUDA
context stays usable (a context with the default limit then iterates normally).

No kernel here faults, traps or spins without a bound: every wait of the three cooperative
schedules (grid barrier, dataflow ready flags, tile flags) counts its polls and leaves when the
count passes the limit, and every thread of the kernel then returns.
"""
import ctypes as C

import pytest

from helpers import small_cascade

pytestmark = pytest.mark.gpu

PRE_UPDATE = ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL", "LUSGS")


@pytest.mark.parametrize("schedule", ["coop", "flow", "tiles"])
def test_sweep_wait_runs_out(gpu_lib, schedule, monkeypatch):
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    monkeypatch.setenv("TRANS_SWEEP", schedule)
    monkeypatch.setenv("TRANS_SWEEP_SPIN", "0")
    monkeypatch.setenv("TRANS_TILE", "4x2x3")
    c, conns, geo, st = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    s = Solver(c, conns, geo, st)
    lib = s.lib
    for name in PRE_UPDATE:
        s.run_stage(name, 1)
    assert lib.trans_run_stage(s.ctx, abi.STAGE_ID["UPDATE"], 1, 1) == abi.TRANS_E_TIMEOUT
    assert b"timed out" in lib.trans_last_error(s.ctx)
    assert lib.trans_update_static_scratch(s.ctx, 1, C.cast(None, C.POINTER(abi.TransNorms))) == abi.TRANS_E_TIMEOUT
    s.close()
    # the device and the library still work: the same case with the default limit
    monkeypatch.delenv("TRANS_SWEEP_SPIN")
    s = Solver(c, conns, geo, st)
    for ki in (1, 2):
        norms = s.iterate(ki)
        assert all(n["nan_flag"] == 0 and n["DRSa"] > 0 for n in norms)
    s.close()


def test_tile_staging_wait_runs_out(gpu_lib, monkeypatch):
    """The mixed path's residual tiles wait on an mbarrier for their TMA copies.  Allowed no
    polls (TRANS_RESID_SPIN=0), every CTA records the error, waits for its copies in flight with
    the default bound (they land; the shared memory they write must outlive them) and returns;
    the UPDATE stage reports TRANS_E_TIMEOUT, and a context with the default limit iterates.
    (The tiled form is selected explicitly: the default is k_face_flux + k_gather.)"""
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    monkeypatch.setenv("TRANS_RESID_TMA", "1")
    monkeypatch.setenv("TRANS_RESID_SPIN", "0")
    c, conns, geo, st = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    c.params.precision = abi.TRANS_MIXED
    s = Solver(c, conns, geo, st)
    lib = s.lib
    for name in PRE_UPDATE:
        s.run_stage(name, 1)
    assert lib.trans_run_stage(s.ctx, abi.STAGE_ID["UPDATE"], 1, 1) == abi.TRANS_E_TIMEOUT
    assert b"residual tile" in lib.trans_last_error(s.ctx)
    s.close()
    monkeypatch.delenv("TRANS_RESID_SPIN")
    s = Solver(c, conns, geo, st)
    for ki in (1, 2):
        norms = s.iterate(ki)
        assert all(n["nan_flag"] == 0 and n["DRSa"] > 0 for n in norms)
    s.close()
