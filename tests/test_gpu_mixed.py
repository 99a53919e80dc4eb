"""Mixed-precision path (FP32 reconstruction, fluxes, SST sources and sweeps; FP64 update,
metrics, time step and norms) against the FP64 path, through the C ABI.

Tolerances (normwise relative, max|mixed - fp64| / max|fp64| per component, per equation group
for the momentum):
  conserved variables, p, T after 20 iterations   5e-5
  residual-norm history (DRSa per iteration)       1e-2 (observed 2.8e-3 on the cascade)
FP32 carries 24 bits (6e-8); the residual subtracts fluxes of similar size, so the FP32 error
of the increment is ~1e-5 of its size early in a run and does not accumulate in the state
beyond a few FP32 ulps per iteration.
"""
import numpy as np
import pytest

from helpers import interior, rel_err, small_annular, small_cascade, small_channel

pytestmark = pytest.mark.gpu

TOL_STATE = 5e-5
TOL_HIST = 1e-2


def _run(case, precision, n):
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    c, conns, geo, st = case
    c.params.precision = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
    s = Solver(c, conns, geo, st)
    hist = [[x["DRSa"] for x in s.iterate(k)] for k in range(1, n + 1)]
    fields = [{f: s.get_field(ib, f) for f in ("V", "PP", "T")} for ib in range(len(c.blocks))]
    s.close()
    return np.array(hist), fields


@pytest.mark.parametrize("make,scheme", [(small_channel, dict(Kind_Spatial=3, Kind_Roe=3)),
                                         (small_channel, dict(Kind_Spatial=2, Kind_Roe=1)),
                                         (small_cascade, dict(Kind_Spatial=3, Kind_Roe=3)),
                                         (small_channel, dict(Kind_Spatial=3, Kind_Roe=3, IF_RK=1, CFL_Sub_start=1.0,
                                                              CFL_Sub_end=1.0)),
                                         (small_channel, dict(Kind_Spatial=1, Kind_Roe=1)),
                                         (small_cascade, dict(Kind_Spatial=4, Kind_Roe=3, F_limiter2=0.05)),
                                         (small_cascade, dict(Kind_Spatial=3, Kind_Roe=3, Kind_Model=2)),
                                         (small_channel, dict(Kind_Spatial=3, Kind_Roe=3, Kind_Hybrid=3, Kind_SubHY=5)),
                                         (small_channel, dict(Kind_Spatial=3, Kind_Roe=3, Kind_RotMod=1)),
                                         (small_annular, dict(Kind_Spatial=3, Kind_Roe=1)),
                                         (small_annular, dict(Kind_Spatial=2, Kind_Roe=1, Kind_RotMod=1))],
                         ids=["channel_mdcd_ausmpw", "channel_muscl_roe", "cascade_mdcd_ausmpw", "channel_rk3_mdcd_ausmpw",
                              "channel_muscl2_roe", "cascade_mdcdhyb_ausmpw", "cascade_mdcd_ausmpw_wd2006",
                              "channel_mdcd_ausmpw_iddes", "channel_mdcd_ausmpw_rc", "annular_rotating_mdcd_roe",
                              "annular_rotating_muscl_roe_rc"])
def test_mixed_tracks_fp64(gpu_lib, make, scheme):
    case = make(**scheme)
    h64, f64 = _run(case, "fp64", 20)
    case = make(**scheme)
    h32, f32 = _run(case, "mixed", 20)
    herr = np.max(np.abs(h32 - h64) / np.abs(h64))
    assert herr <= TOL_HIST, f"residual history differs by {herr:.3e}"
    for ib, b in enumerate(case[0].blocks):
        m = interior(b.dims)
        for name in ("PP", "T"):
            err = np.max(rel_err(f32[ib][name], f64[ib][name], m))
            assert err <= TOL_STATE, f"block {b.id} {name}: {err:.3e}"
        # conserved variables, normwise per equation group: density, momentum (the spanwise
        # component of these nearly two-dimensional flows is tiny on its own), energy, k, omega
        for grp in ((0,), (1, 2, 3), (4,), (5,), (6,)):
            scale = max(np.max(np.abs(f64[ib]["V"][q][m])) for q in grp)
            if scale == 0.0:
                continue
            err = max(np.max(np.abs(f32[ib]["V"][q][m] - f64[ib]["V"][q][m])) for q in grp) / scale
            assert err <= TOL_STATE, f"block {b.id} V{grp}: {err:.3e}"


def test_mixed_residual_field_readback(gpu_lib):
    """D is held in FP32 by the mixed path; trans_get_field(TRANS_D) returns it widened."""
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_channel(Kind_Spatial=3, Kind_Roe=3)
    c.params.precision = abi.TRANS_MIXED
    s = Solver(c, conns, geo, st)
    for stage in ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL"):
        s.run_stage(stage, 1)
    D32 = s.get_field(0, "D")
    s.close()
    c, conns, geo, st = small_channel(Kind_Spatial=3, Kind_Roe=3)
    s = Solver(c, conns, geo, st)
    for stage in ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL"):
        s.run_stage(stage, 1)
    D64 = s.get_field(0, "D")
    s.close()
    m = interior(c.blocks[0].dims)
    # scale: the largest residual of the same equation group (the spanwise-momentum residual
    # of this channel is tiny on its own)
    groups = [(0,), (1, 2, 3), (4,)]
    for g in groups:
        scale = max(np.max(np.abs(D64[q][m])) for q in g)
        for q in g:
            err = np.max(np.abs(D32[q][m] - D64[q][m])) / scale
            assert err < 2e-4, (q, err)
