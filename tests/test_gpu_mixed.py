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


def _first_residual(case, precision, env="1"):
    """D after the first iteration's residual stage of a context of the given precision,
    created with the given TRANS_RESID_TMA setting, and the kernel classes that ran."""
    import os
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    c, conns, geo, st = case
    c.params.precision = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
    old = os.environ.get("TRANS_RESID_TMA")
    os.environ["TRANS_RESID_TMA"] = env
    try:
        s = Solver(c, conns, geo, st)
    finally:
        if old is None:
            del os.environ["TRANS_RESID_TMA"]
        else:
            os.environ["TRANS_RESID_TMA"] = old
    for stage in ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL"):
        s.run_stage(stage, 1)
    D = [s.get_field(ib, "D") for ib in range(len(c.blocks))]
    s.iterate(2)
    import bench
    names = set(bench.kernel_times(s, 3))
    s.close()
    return D, names


@pytest.mark.parametrize("make,scheme", [(small_channel, dict(Kind_Spatial=3, Kind_Roe=3)),
                                         (small_channel, dict(Kind_Spatial=2, Kind_Roe=1)),
                                         (small_cascade, dict(Kind_Spatial=3, Kind_Roe=3)),
                                         (small_cascade, dict(Kind_Spatial=4, Kind_Roe=3, F_limiter2=0.05)),
                                         (small_annular, dict(Kind_Spatial=3, Kind_Roe=1))],
                         ids=["channel_mdcd_ausmpw", "channel_muscl_roe", "cascade_mdcd_ausmpw", "cascade_mdcdhyb_ausmpw",
                              "annular_rotating_mdcd_roe"])
def test_tma_tiles_match_face_flux_kernels(gpu_lib, make, scheme):
    """The mixed path's residual from TMA-staged shared-memory tiles (k_resid_tma,
    TRANS_RESID_TMA=1) against its residual from k_face_flux<float> + k_gather<float> (the
    default, TRANS_RESID_TMA=0), both
    against the FP64 residual: the same FP32 face arithmetic, summed per direction instead of in
    the gather's order.  D is a difference of fluxes many times its size, so FP32 rounding of the
    fluxes shows in D well above FP32's own precision (1e-2 of the largest density residual of
    a cascade block at the uniform initial state, where the fluxes nearly cancel); the tiled path
    must be as close to FP64 as the gather path (within 3x its error, plus 1e-6 of the largest
    |D|), per equation group and block."""
    D_t, names_t = _first_residual(make(**scheme), "mixed", "1")
    D_g, names_g = _first_residual(make(**scheme), "mixed", "0")
    D_64, _ = _first_residual(make(**scheme), "fp64")
    assert "k_resid_tma" in names_t and "k_face_flux" not in names_t and "k_gather" not in names_t
    assert "k_face_flux" in names_g and "k_resid_tma" not in names_g
    case = make(**scheme)
    for ib, b in enumerate(case[0].blocks):
        m = interior(b.dims)
        for grp in ((0,), (1, 2, 3), (4,), (5,), (6,)):
            scale = max(np.max(np.abs(D_64[ib][q][m])) for q in grp)
            if scale == 0.0:
                continue
            e_t = max(np.max(np.abs(D_t[ib][q][m] - D_64[ib][q][m])) for q in grp) / scale
            e_g = max(np.max(np.abs(D_g[ib][q][m] - D_64[ib][q][m])) for q in grp) / scale
            assert e_t <= 3.0 * e_g + 1e-6, f"block {b.id} D{grp}: tiled {e_t:.3e}, gather {e_g:.3e}"


def test_residual_form_tuner_on_request(gpu_lib, monkeypatch):
    """TRANS_RESID_TMA=auto: the context times both residual forms on its first residual,
    reports both times in trans_tuning and keeps one of them; without it the gather form runs
    and nothing is timed."""
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    for env, timed in (("auto", True), (None, False)):
        if env:
            monkeypatch.setenv("TRANS_RESID_TMA", env)
        else:
            monkeypatch.delenv("TRANS_RESID_TMA", raising=False)
        c, conns, geo, st = small_cascade(Kind_Spatial=3, Kind_Roe=3)
        c.params.precision = abi.TRANS_MIXED
        s = Solver(c, conns, geo, st)
        s.iterate(1)
        tuning = s.lib.trans_tuning(s.ctx).decode()
        s.close()
        assert ("tma:" in tuning and "gather:" in tuning) == timed, tuning
        assert "residual=tma" in tuning or "residual=gather" in tuning, tuning
        if not timed:
            assert "residual=gather" in tuning, tuning
