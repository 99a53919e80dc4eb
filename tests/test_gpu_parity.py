"""GPU FP64 path against the CPU oracle, through the C ABI.

Tolerance: 1e-11 relative (normwise per component, max|gpu-oracle| / max|oracle|) on every
per-cell quantity and on the residual history, the bar the plain FP64 path is held to.
"""
import numpy as np
import pytest

from helpers import bit_equal_fraction, face_ghosts, interior, rel_err, small_channel

TOL = 1e-11

pytestmark = pytest.mark.gpu


def _pair(c, conns, geo, st):
    from oracle.oracle import OracleSolver
    from trans_gb300.solver import Solver
    return Solver(c, conns, geo, st), OracleSolver(c, conns, geo, st)


STAGE_FIELDS = {
    "SPECRAD": [("RDS", "int"), ("DTM", "int")],
    "BC_STATE": [("V", "ghost"), ("PP", "ghost"), ("T", "ghost"), ("RMIU", "ghost")],
    "GRADIENT": [("DQDXYZ", "int"), ("SHOCK", "int"), ("SHOCK", "ghost")],
    "BC_GRAD": [("DQDXYZ", "ghost1")],
    "RESIDUAL": [("D", "int")],
    "LUSGS": [("D", "int")],
    "UPDATE": [("V", "int"), ("PP", "int"), ("T", "int"), ("RMIU", "int")],
}


def _mask(kind, dims):
    if kind == "int":
        return interior(dims)
    if kind == "ghost":
        return face_ghosts(dims, 3)
    return face_ghosts(dims, 1)


# Kind_Spatial 1 = MUSCL2 limiter, 4 = MDCD/MUSCL hybrid; F_limiter2 = 0.05 puts the hybrid switch
# inside the sensor's range on these grids (a mix of MDCD and MUSCL faces)
# Kind_Model 2 = the WD+2006 k-omega model in place of SST
SCHEMES = [dict(Kind_Spatial=2, Kind_Roe=1), dict(Kind_Spatial=3, Kind_Roe=3), dict(Kind_Spatial=1, Kind_Roe=1),
           dict(Kind_Spatial=4, Kind_Roe=3, F_limiter2=0.05), dict(Kind_Spatial=3, Kind_Roe=3, Kind_Model=2),
           dict(Kind_Spatial=2, Kind_Roe=2), dict(Kind_Spatial=3, Kind_Roe=2)]
SCHEME_IDS = ["muscl_roe", "mdcd_ausmpw", "muscl2_roe", "mdcdhyb_ausmpw", "mdcd_ausmpw_wd2006", "muscl_roerot",
              "mdcd_roerot"]


@pytest.mark.parametrize("scheme", SCHEMES, ids=SCHEME_IDS)
def test_stage_by_stage(gpu_lib, scheme):
    c, conns, geo, st = small_channel(**scheme)
    g, o = _pair(c, conns, geo, st)
    dims = c.blocks[0].dims
    for ki in (1, 2):
        for stage, fields in STAGE_FIELDS.items():
            g.run_stage(stage, ki)
            o.run_stage(stage, ki)
            for name, mk in fields:
                m = _mask(mk, dims)
                a, b = g.get_field(0, name), o.get_field(0, name)
                err = np.max(rel_err(a, b, m))
                assert err <= TOL, f"iteration {ki} stage {stage} field {name}/{mk}: rel err {err:.3e}"
        g.run_stage("UPDATE_U", ki)
        o.run_stage("UPDATE_U", ki)


@pytest.mark.parametrize("scheme", SCHEMES, ids=SCHEME_IDS)
def test_iterations_and_residual_history(gpu_lib, scheme):
    """100 outer iterations: the state stays bit-identical to the oracle's (the FP64 kernels and
    the oracle round every operation alike), the residual norms agree to summation order."""
    c, conns, geo, st = small_channel(**scheme)
    g, o = _pair(c, conns, geo, st)
    dims = c.blocks[0].dims
    m = interior(dims)
    hg, ho = [], []
    for ki in range(1, 101):
        ng = g.iterate(ki)
        no = o.iterate(ki)
        hg.append(ng[0]["DRSa"]); ho.append(no[0]["DRSa"])
    hist = np.max(np.abs(np.array(hg) - np.array(ho)) / np.abs(np.array(ho)))
    assert hist <= TOL, f"L2 residual history differs by {hist:.3e}"
    for name in ("V", "PP", "T", "RMIU"):
        a, b = g.get_field(0, name), o.get_field(0, name)
        err = np.max(rel_err(a, b, m))
        assert err <= TOL, f"{name} after 100 iterations: {err:.3e}"
        frac = bit_equal_fraction(a, b, m)
        assert frac == 1.0, f"{name}: only {frac:.6f} of the values are bit-identical"


def test_bitwise_agreement_first_residual(gpu_lib):
    """Without fused multiply-add, and with exp/tanh/pow evaluated by the same methods on both
    sides, the FP64 residual matches the oracle bit for bit."""
    c, conns, geo, st = small_channel(Kind_Spatial=3, Kind_Roe=3)
    g, o = _pair(c, conns, geo, st)
    for s in ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL"):
        g.run_stage(s, 1)
        o.run_stage(s, 1)
    frac = bit_equal_fraction(g.get_field(0, "D"), o.get_field(0, "D"), interior(c.blocks[0].dims))
    assert frac == 1.0, f"only {frac:.6f} of residual values are bit-identical"


@pytest.mark.parametrize("scheme", SCHEMES, ids=SCHEME_IDS)
def test_cascade_multiblock_bitwise(gpu_lib, scheme):
    """Five blocks with 1-to-1 interfaces (O-cut, pitch periodicity, partial faces with
    reversed index direction), inlet, outlet recurrence and walls: 12 iterations stay
    bit-identical to the oracle in every block."""
    from helpers import small_cascade
    c, conns, geo, st = small_cascade(**scheme)
    g, o = _pair(c, conns, geo, st)
    for ki in range(1, 13):
        ng = g.iterate(ki)
        no = o.iterate(ki)
        for b in range(len(c.blocks)):
            assert abs(ng[b]["DRSa"] - no[b]["DRSa"]) <= TOL * no[b]["DRSa"]
    for ib, b in enumerate(c.blocks):
        m = interior(b.dims)
        for name in ("V", "PP", "T", "RMIU"):
            frac = bit_equal_fraction(g.get_field(ib, name), o.get_field(ib, name), m)
            assert frac == 1.0, f"block {b.id} {name}: {frac:.6f} bit-identical"


RK3 = dict(Kind_Spatial=3, Kind_Roe=3, IF_RK=1, CFL_Sub_start=1.0, CFL_Sub_end=1.0)


def test_runge_kutta_stages_bitwise(gpu_lib):
    """IF_RK = 1 (main.F90:152-161): every SSP-RK3 stage -- Wt2, the mean-flow stage update with
    its norms, the k-omega LU-SGS increments on the new state and TIME_RK_V_Update_New --
    bit-identical to the oracle, stage by stage, over two outer iterations."""
    c, conns, geo, st = small_channel(**RK3)
    g, o = _pair(c, conns, geo, st)
    m = interior(c.blocks[0].dims)
    for ki in (1, 2):
        for itr in (1, 2, 3):
            for stage in ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL", "LUSGS"):
                g.run_stage(stage, ki, itr)
                o.run_stage(stage, ki, itr)
            for name in ("WT2", "V", "D"):
                a, b = g.get_field(0, name), o.get_field(0, name)
                frac = bit_equal_fraction(a, b, m)
                assert frac == 1.0, f"iteration {ki} stage {itr} {name} after LUSGS: {frac:.6f} bit-identical"
            g.run_stage("UPDATE", ki, itr)
            o.run_stage("UPDATE", ki, itr)
            for name in ("V", "PP", "T", "RMIU"):
                frac = bit_equal_fraction(g.get_field(0, name), o.get_field(0, name), m)
                assert frac == 1.0, f"iteration {ki} stage {itr} {name} after UPDATE: {frac:.6f} bit-identical"
            ng, no = g.norms(), o.norms()
            for key in ("DRSa", "DRSk", "DRSo"):
                assert abs(ng[0][key] - no[0][key]) <= TOL * no[0][key], (ki, itr, key)
            assert ng[0]["DUa"] == no[0]["DUa"] and ng[0]["Ima"] == no[0]["Ima"]
        g.run_stage("UPDATE_U", ki, 3)
        o.run_stage("UPDATE_U", ki, 3)


@pytest.mark.parametrize("kind", ["channel", "cascade", "channel_wd2006"])
def test_runge_kutta_iterations_bitwise(gpu_lib, kind):
    """Runge-Kutta outer iterations through trans_iterate (3 stages each): the state stays
    bit-identical to the oracle's, the norms of every block agree to summation order."""
    from helpers import small_cascade
    if kind == "channel_wd2006":
        c, conns, geo, st = small_channel(**RK3, Kind_Model=2)
    else:
        c, conns, geo, st = small_channel(**RK3) if kind == "channel" else small_cascade(**RK3)
    g, o = _pair(c, conns, geo, st)
    n = 8 if kind == "cascade" else 30
    for ki in range(1, n + 1):
        ng = g.iterate(ki)
        no = o.iterate(ki)
        for b in range(len(c.blocks)):
            for key in ("DRSa", "DRSk", "DRSo"):
                assert abs(ng[b][key] - no[b][key]) <= TOL * no[b][key], (ki, b, key)
    for ib, b in enumerate(c.blocks):
        m = interior(b.dims)
        for name in ("V", "PP", "T", "RMIU", "WT2"):
            frac = bit_equal_fraction(g.get_field(ib, name), o.get_field(ib, name), m)
            assert frac == 1.0, f"block {b.id} {name}: {frac:.6f} bit-identical"


def test_square_cylinder_des_bitwise(gpu_lib):
    """The square-cylinder DES configuration (O-block wrapping through a self 1-to-1 cut,
    periodic span, far field, dual time with 10 sub-iterations per step) on a coarse grid:
    three physical steps bit-identical to the oracle."""
    from trans_gb300 import cases
    from trans_gb300 import case as CS
    c = cases.square_cylinder(ni=33, nj=17, nk=9)
    conns, geo = CS.compute_geometry(c)
    st = CS.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    g, o = _pair(c, conns, geo, st)
    for ki in range(1, 4):
        ng = g.iterate(ki)
        no = o.iterate(ki)
        for key in ("DRSa", "DRSk", "DRSo"):
            assert abs(ng[0][key] - no[0][key]) <= TOL * no[0][key], (ki, key)
    m = interior(c.blocks[0].dims)
    for name in ("V", "PP", "T", "RMIU"):
        frac = bit_equal_fraction(g.get_field(0, name), o.get_field(0, name), m)
        assert frac == 1.0, f"{name}: {frac:.6f} bit-identical"


def _goldens():
    import os
    d = os.path.join(os.path.dirname(__file__), "golden")
    return sorted(f for f in os.listdir(d) if f.endswith(".json"))


@pytest.mark.parametrize("name", _goldens())
def test_gpu_against_golden_vectors(gpu_lib, name):
    """The CUDA path reproduces the committed golden vectors: residual history of every block
    over ten iterations and probed conserved variables (tolerance of the fixtures, 1e-12: the
    inputs are bit-identical on every CPU, only the norm summation order differs)."""
    import json
    import os
    from trans_gb300.solver import Solver
    from test_oracle import GOLD_TOL, golden_case
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", name)))
    from helpers import inputs_digest
    c, conns, geo, st = golden_case(g)
    assert inputs_digest(c, geo, st) == g["inputs_sha256"], "host set-up is not bit-reproducible"
    s = Solver(c, conns, geo, st)
    hist = [[n["DRSa"] for n in s.iterate(k)] for k in range(1, len(g["DRSa"]) + 1)]
    np.testing.assert_allclose(hist, g["DRSa"], rtol=GOLD_TOL)
    for p in g["probes"]:
        V = s.get_field(p["block"], "V")
        i, j, k = p["at"]
        np.testing.assert_allclose([V[L, i + 2, j + 2, k + 2] for L in range(7)], p["V"], rtol=GOLD_TOL)
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sweep_schedules_agree_bitwise(gpu_lib, precision, monkeypatch):
    """The hyperplane-per-launch schedule, the single cooperative launch with grid barriers, the
    dataflow schedule, the tiled wavefront (two tile shapes), each with the lane-major and the
    warp-per-component thread mapping (FP64), the chaining, prefetch and CTA-size variants of the
    hyperplane launches, the mixed path's cluster-barrier schedule (one thread-block cluster per
    block) and two-plane schedule (the positions of a plane recomputed by each neighbour on the
    next; the FP64 path runs planes for both), and the tuner's pick compute every DeltaQ with
    the same operations: states after 6 iterations are bit-identical."""
    from helpers import small_cascade
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    out = {}
    modes = ("planes", "planes_unchained", "coop", "flow", "tiles", "tiles_4x2x3", "planes_wpc", "planes_unchained_wpc",
             "coop_wpc", "tiles_4x2x3_wpc", "planes_pf2", "planes_wpc_pf1", "planes_early_cta32", "planes_early_pf2_cta64",
             "clusters", "clusters_pf2", "pairs", "pairs_unchained", "pairs_early_cta32", "pairs_early_pf1_cta128", "auto")
    for mode in modes:
        parts = mode.split("_")
        monkeypatch.setenv("TRANS_SWEEP", parts[0])
        monkeypatch.setenv("TRANS_PDL", "0" if "unchained" in parts else ("2" if "early" in parts else "1"))
        monkeypatch.setenv("TRANS_SWEEP_CTA", next((x[3:] for x in parts if x.startswith("cta")), "0"))
        monkeypatch.setenv("TRANS_TILE", next((x for x in parts if "x" in x), "8x8x8"))
        monkeypatch.setenv("TRANS_SWEEP_MAP", "wpc" if "wpc" in parts else "lane")
        monkeypatch.setenv("TRANS_SWEEP_PF", next((x[2:] for x in parts if x.startswith("pf")), "0"))
        c, conns, geo, st = small_cascade(Kind_Spatial=3, Kind_Roe=3)
        c.params.precision = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
        s = Solver(c, conns, geo, st)
        for ki in range(1, 7):
            s.iterate(ki)
        out[mode] = [s.get_field(ib, "V") for ib in range(len(c.blocks))]
        s.close()
    for mode in modes[1:]:
        for ib in range(len(out["planes"])):
            m = interior(c.blocks[ib].dims)
            assert bit_equal_fraction(out[mode][ib], out["planes"][ib], m) == 1.0, (mode, ib)


def test_pair_sweeps_runge_kutta_bitwise(gpu_lib, monkeypatch):
    """Mixed path, SSP-RK3 (the sweeps carry only k and omega, the other components pass through
    the two DeltaQ arrays unchanged): the two-plane schedule equals one launch per plane bit for
    bit, on the channel and on the five-block cascade."""
    from helpers import small_cascade
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    for make in (small_channel, small_cascade):
        out = {}
        for mode in ("planes", "pairs"):
            monkeypatch.setenv("TRANS_SWEEP", mode)
            c, conns, geo, st = make(Kind_Spatial=3, Kind_Roe=3, IF_RK=1, CFL_Sub_start=1.0, CFL_Sub_end=1.0)
            c.params.precision = abi.TRANS_MIXED
            s = Solver(c, conns, geo, st)
            for ki in range(1, 4):
                s.iterate(ki)
            out[mode] = [s.get_field(ib, "V") for ib in range(len(c.blocks))]
            s.close()
        for ib in range(len(out["planes"])):
            m = interior(c.blocks[ib].dims)
            assert bit_equal_fraction(out["pairs"][ib], out["planes"][ib], m) == 1.0, (make.__name__, ib)


def test_long_run_field_parity(gpu_lib):
    """1500 iterations (the residual has dropped ~3 orders and settled): fields within 1e-8 of
    the oracle (the bar for the converged field; they stay bit-identical in practice)."""
    c, conns, geo, st = small_channel(Kind_Spatial=3, Kind_Roe=3)
    g, o = _pair(c, conns, geo, st)
    for ki in range(1, 1501):
        g.iterate(ki)
        o.iterate(ki)
    m = interior(c.blocks[0].dims)
    for name in ("V", "PP", "T", "RMIU"):
        err = np.max(rel_err(g.get_field(0, name), o.get_field(0, name), m))
        assert err <= 1e-8, f"{name}: {err:.3e}"


def test_des_dual_time_bitwise(gpu_lib):
    """SST-DES length scale (Kind_Hybrid=3, loop-carried F1 of the previous cell) with dual time
    stepping (Kind_Dual=2, 3 sub-iterations per physical step): bit-identical to the oracle."""
    c, conns, geo, st = small_channel(Kind_Spatial=3, Kind_Roe=3, Kind_Hybrid=3, Kind_SubHY=0, Kchld=3,
                                      DT_LUSGS_Main=0.05)
    g, o = _pair(c, conns, geo, st)
    m = interior(c.blocks[0].dims)
    for ki in range(1, 6):
        ng, no = g.iterate(ki), o.iterate(ki)
        assert abs(ng[0]["DRSa"] - no[0]["DRSa"]) <= TOL * no[0]["DRSa"]
    for name in ("V", "PP", "T", "RMIU", "WT0", "WT1"):
        frac = bit_equal_fraction(g.get_field(0, name), o.get_field(0, name), m)
        assert frac == 1.0, f"{name}: {frac:.6f} bit-identical"


def test_rotational_periodic_annulus_bitwise(gpu_lib):
    """An annular sector whose periodic faces rotate (v, w) and the velocity gradients by
    +-10 degrees at the 1-to-1 interface (BC/BC_P2P.F90:69-181): 12 iterations bit-identical
    to the oracle."""
    from trans_gb300 import case as CS
    from trans_gb300 import cases
    c = cases.annular_sector()
    conns, geo = CS.compute_geometry(c)
    assert sorted(round(cn.rotateAngle, 6) for cn in conns[1] if cn.BCType == 9) == [-0.174533, 0.174533]
    st = CS.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    g, o = _pair(c, conns, geo, st)
    for ki in range(1, 13):
        ng, no = g.iterate(ki), o.iterate(ki)
        assert abs(ng[0]["DRSa"] - no[0]["DRSa"]) <= TOL * no[0]["DRSa"]
    m = interior(c.blocks[0].dims)
    for name in ("V", "PP", "T", "RMIU"):
        frac = bit_equal_fraction(g.get_field(0, name), o.get_field(0, name), m)
        assert frac == 1.0, f"{name}: {frac:.6f} bit-identical"
