"""GPU FP64 path against the CPU oracle on the configurations and switches the scheme-set tests
do not reach, through the C ABI:

- the channel bump at its benchmark size (97x49x9 nodes, 36,864 cells) for 100 iterations;
- the five-block cascade at the benchmark's block sizes (1,966,080 cells) for 3 iterations;
- the DDES shielding functions of Time/Hybrid_function.F90:1-38 (Kind_SubHY = 1, 2, 3) under
  the DES length scale of Time/TURBTWO_TIME_LUSGS_SST.F90:192-213, and IDDES (Kind_SubHY = 5);
- Suzen's compressibility correction (IF_Comppress = 1, Time/TURBTWO_TIME_LUSGS_SST.F90:339-397);
- the fixed-transition switch (If_fix_Transition = 1: no k source upstream of Trans_location,
  Time/TURBTWO_TIME_LUSGS_SST.F90:291-293);
- a symmetry plane (kind 3, BC/BC_Symm.F90:42-121), stage by stage and over iterations;
- low-Mach preconditioning, RC correction, and a rotating frame (omega(1) != 0) on the
  annular sector with every spatial and flux scheme.

Bar: bit-identical states (the FP64 kernels and the oracle round every operation alike) and
the residual history within 1e-11 relative (summation order).
"""
import numpy as np
import pytest

from helpers import G, bit_equal_fraction, face_ghosts, interior, rel_err, small_channel

TOL = 1e-11

pytestmark = pytest.mark.gpu


def _pair(c, conns, geo, st, threads=None):
    from oracle.oracle import OracleSolver, load
    from trans_gb300.solver import Solver
    if threads:
        load().oracle_set_threads(threads)
    return Solver(c, conns, geo, st), OracleSolver(c, conns, geo, st)


def _run_bitwise(c, conns, geo, st, iters, fields=("V", "PP", "T", "RMIU"), threads=None):
    g, o = _pair(c, conns, geo, st, threads)
    hg, ho = [], []
    for ki in range(1, iters + 1):
        ng, no = g.iterate(ki), o.iterate(ki)
        hg.append([n["DRSa"] for n in ng]); ho.append([n["DRSa"] for n in no])
    hg, ho = np.array(hg), np.array(ho)
    hist = np.max(np.abs(hg - ho) / np.abs(ho))
    assert hist <= TOL, f"residual history differs by {hist:.3e}"
    for ib, b in enumerate(c.blocks):
        m = interior(b.dims)
        for name in fields:
            a, r = g.get_field(ib, name), o.get_field(ib, name)
            frac = bit_equal_fraction(a, r, m)
            assert frac == 1.0, f"block {b.id} {name}: {frac:.6f} bit-identical, rel err {np.max(rel_err(a, r, m)):.3e}"
    g.close(); o.close()
    return hg


def test_channel_benchmark_size_100_iterations(gpu_lib):
    """The channel bump as the benchmark states it: 97x49x9 nodes, MUSCL + Roe, SST, CFL 5."""
    from trans_gb300 import case as CS
    from trans_gb300 import cases
    c = cases.channel_bump()
    assert c.blocks[0].dims == (97, 49, 9)
    conns, geo = CS.compute_geometry(c)
    st = CS.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    hist = _run_bitwise(c, conns, geo, st, 100)
    assert np.all(np.isfinite(hist))


def test_cascade_benchmark_size_3_iterations(gpu_lib):
    """The benchmarked cascade at full size (O 257x49x65, H 65x97x65, passage 97x33x65;
    MDCD + AUSMPW+, SST, CFL 10): 3 iterations bit-identical in every block."""
    from trans_gb300 import case as CS
    from trans_gb300 import cases
    from trans_gb300.solver import device_block_metrics
    c = cases.cascade(**cases.CASCADE_CONFIG2)
    conns, geo = CS.compute_geometry(c, metrics_fn=device_block_metrics())
    st = CS.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    _run_bitwise(c, conns, geo, st, 3, threads=8)


DES = dict(Kind_Spatial=3, Kind_Roe=3, Kind_Hybrid=3)


@pytest.mark.parametrize("subhy", [1, 2, 3, 5])
def test_ddes_shielding_functions(gpu_lib, subhy):
    """Kind_Hybrid = 3 with Menter's F1 (1), Menter's F2 (2) and Spalart's F1 (3) shielding, and
    IDDES (5): its length scale from fd/fe (Time/Hybrid_function.F90:43-105) and its own k
    destruction and diagonal (Time/TURBTWO_TIME_LUSGS_SST.F90:218-252, 299-310)."""
    c, conns, geo, st = small_channel(Kind_SubHY=subhy, **DES)
    _run_bitwise(c, conns, geo, st, 20)


def test_iddes_with_compressibility_and_transition(gpu_lib):
    """IDDES with Suzen's correction of its destruction (:354-366) and the fixed-transition
    switch inside the IDDES branch."""
    from trans_gb300 import case as CS
    from trans_gb300 import cases
    probe = cases.channel_bump(ni=25, nj=17, nk=6)
    c = cases.channel_bump(ni=25, nj=17, nk=6, Kind_SubHY=5, IF_Comppress=1, If_fix_Transition=1,
                           Trans_location=0.5 / probe.params.Alscale, **DES)
    conns, geo = CS.compute_geometry(c)
    st = CS.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    _run_bitwise(c, conns, geo, st, 20)


def test_undefined_shielding_switch_rejected(gpu_lib):
    """Kind_SubHY = 4 has no branch in FSST (its result would be undefined): refused."""
    from trans_gb300 import abi
    from trans_gb300.solver import Solver, SolverError
    c, conns, geo, st = small_channel(Kind_SubHY=4, **DES)
    with pytest.raises(SolverError, match=str(abi.TRANS_E_ARG)):
        Solver(c, conns, geo, st)


@pytest.mark.parametrize("hybrid", [0, 3], ids=["rans", "des"])
def test_suzen_compressibility_correction(gpu_lib, hybrid):
    c, conns, geo, st = small_channel(Kind_Spatial=3, Kind_Roe=3, IF_Comppress=1, Kind_Hybrid=hybrid)
    _run_bitwise(c, conns, geo, st, 20)


def test_fixed_transition(gpu_lib):
    """If_fix_Transition = 1 with Trans_location halfway along the channel: the k source is
    zero in the cells whose centre lies upstream of it."""
    from trans_gb300 import case as CS
    from trans_gb300 import cases
    probe = cases.channel_bump(ni=25, nj=17, nk=6)
    c = cases.channel_bump(ni=25, nj=17, nk=6, Kind_Spatial=3, Kind_Roe=3, If_fix_Transition=1,
                           Trans_location=0.5 / probe.params.Alscale)
    conns, geo = CS.compute_geometry(c)
    xc = geo[c.blocks[0].id]["XC"][interior(c.blocks[0].dims)]
    assert np.any(xc < c.params.Trans_location) and np.any(xc > c.params.Trans_location)
    st = CS.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    _run_bitwise(c, conns, geo, st, 20)


def _symmetry_case():
    """The channel with a symmetry plane on top.  BC_Symm sets every ghost value of the three
    layers except the density of layer 2 (BC/BC_Symm.F90:70-79), which keeps what the restart
    held: the ghost density is filled with the free-stream value, as in a restart of a run."""
    c, conns, geo, st = small_channel(Kind_Spatial=2, Kind_Roe=1, top=3)
    for b in c.blocks:
        V = st[b.id]["V"]
        m = ~interior(b.dims)
        V[0][m] = 1.0
    return c, conns, geo, st


def _ghost_mismatches(a, b, dims):
    """(face, layer, component, count, sample gpu, sample oracle) of the face ghosts that differ
    bit for bit (face 0..5 = i-min, i-max, j-min, j-max, k-min, k-max)."""
    ni, nj, nk = dims
    out = []
    a2 = a.reshape((-1,) + a.shape[-3:])
    b2 = b.reshape((-1,) + b.shape[-3:])
    I, J, K = slice(G + 1, G + ni), slice(G + 1, G + nj), slice(G + 1, G + nk)
    for L in range(1, 4):
        sl = [(G + 1 - L, J, K), (G + ni - 1 + L, J, K), (I, G + 1 - L, K), (I, G + nj - 1 + L, K),
              (I, J, G + 1 - L), (I, J, G + nk - 1 + L)]
        for f, s in enumerate(sl):
            for q in range(a2.shape[0]):
                x, y = a2[q][s].ravel(), b2[q][s].ravel()
                bad = x.view(np.int64) != y.view(np.int64)
                if np.any(bad):
                    k = int(np.argmax(bad))
                    out.append((f, L, q, int(bad.sum()), float(x[k]), float(y[k])))
    return out


def test_symmetry_plane_bc_state_stage(gpu_lib):
    """BC_STATE on the three ghost layers of every face (the symmetry plane among them), then
    the gradients and their ghost copies, against the oracle."""
    c, conns, geo, st = _symmetry_case()
    g, o = _pair(c, conns, geo, st)
    dims = c.blocks[0].dims
    ni, nj, nk = dims
    top = np.zeros((ni + 5, nj + 5, nk + 5), bool, order="F")
    top[G + 1:G + ni, G + nj:G + nj + 3, G + 1:G + nk] = True
    for ki in (1, 2):
        for stage in ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL", "LUSGS", "UPDATE", "UPDATE_U"):
            g.run_stage(stage, ki)
            o.run_stage(stage, ki)
            if stage == "BC_STATE":
                for name in ("V", "PP", "T", "RMIU"):
                    a, b = g.get_field(0, name), o.get_field(0, name)
                    assert bit_equal_fraction(a, b, top) == 1.0, (ki, name)
                    bad = _ghost_mismatches(a, b, dims)
                    assert not bad, (ki, name, bad[:12])
                # the mirror: the layer-1 ghost's momentum is the first interior cell's reflected
                # about the unit normal of the face BC_Symm reads, i + IJKAdd with IJKAdd = -1 on a
                # max face (Input/PLOT3DReadInit.F90:235): the first interior face, which follows
                # the bump below the flat top (BC/BC_Symm.F90:46-49, 59-63)
                V = g.get_field(0, "V")
                gb = geo[c.blocks[0].id]
                n = np.stack([gb["SD"][1, q, G + 1:G + ni, G + nj - 1, G + 1:G + nk] for q in range(3)])
                n = n / gb["GRAD"][1, G + 1:G + ni, G + nj - 1, G + 1:G + nk]
                rho = V[0][G + 1:G + ni, G + nj - 1, G + 1:G + nk]
                m_in = np.stack([V[q][G + 1:G + ni, G + nj - 1, G + 1:G + nk] for q in (1, 2, 3)])
                vc = np.sum(n * m_in / rho, axis=0)
                want = m_in - 2.0 * n * vc * rho
                got = np.stack([V[q][G + 1:G + ni, G + nj, G + 1:G + nk] for q in (1, 2, 3)])
                assert np.allclose(got, want, rtol=1e-12, atol=1e-14), (ki, np.max(np.abs(got - want)))
            if stage == "BC_GRAD":
                a, b = g.get_field(0, "DQDXYZ"), o.get_field(0, "DQDXYZ")
                assert bit_equal_fraction(a, b, face_ghosts(dims, 1)) == 1.0, ki
    g.close(); o.close()


def test_symmetry_plane_iterations(gpu_lib):
    c, conns, geo, st = _symmetry_case()
    _run_bitwise(c, conns, geo, st, 30)


def _precond_channel(XM, **sw):
    from trans_gb300 import case as CS
    from trans_gb300 import cases
    c = cases.channel_bump(ni=25, nj=17, nk=6, XM=XM, IF_Precondition=1, **sw)
    conns, geo = CS.compute_geometry(c)
    st = CS.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    return c, conns, geo, st


@pytest.mark.parametrize("scheme", [dict(Kind_Spatial=2, Kind_Roe=1), dict(Kind_Spatial=3, Kind_Roe=3)],
                         ids=["muscl_roe", "mdcd_ausmpw"])
def test_preconditioning_iterations(gpu_lib, scheme):
    """Low-Mach preconditioning (IF_Precondition = 1, Common/UTIL_Precond_Funcs.F90): the spectral
    radius (Time/SpectralRadius.F90:91-127), the Roe dissipation (Space/CONVECT_Roe_Original.F90:
    319-331), PrecondDW of the right-hand side and of every neighbour term of both sweeps
    (Time/TIME_LUSGS.F90:113-160, 235-248) and the conservative update (Time/TIME_Update_V.F90:
    580-607), 20 iterations at M 0.3, bit-identical."""
    c, conns, geo, st = _precond_channel(0.3, **scheme)
    _run_bitwise(c, conns, geo, st, 20)


def test_preconditioning_stage_by_stage(gpu_lib):
    c, conns, geo, st = _precond_channel(0.3, Kind_Spatial=2, Kind_Roe=1)
    g, o = _pair(c, conns, geo, st)
    m = interior(c.blocks[0].dims)
    for ki in (1, 2):
        for stage, fields in (("SPECRAD", ("RDS", "DTM")), ("BC_STATE", ()), ("GRADIENT", ()), ("BC_GRAD", ()),
                              ("RESIDUAL", ("D",)), ("LUSGS", ("D",)), ("UPDATE", ("V", "PP", "T", "RMIU")),
                              ("UPDATE_U", ())):
            g.run_stage(stage, ki)
            o.run_stage(stage, ki)
            for f in fields:
                assert bit_equal_fraction(g.get_field(0, f), o.get_field(0, f), m) == 1.0, (ki, stage, f)
    g.close(); o.close()


def test_preconditioning_low_mach_first_iterations(gpu_lib):
    """At M 0.1 (ubetac2 near 3 M^2) the first iterations, bit-identical."""
    c, conns, geo, st = _precond_channel(0.1, Kind_Spatial=2, Kind_Roe=1)
    _run_bitwise(c, conns, geo, st, 6)


def test_preconditioning_fp64_path_only(gpu_lib):
    from trans_gb300 import abi
    from trans_gb300.solver import Solver, SolverError
    c, conns, geo, st = _precond_channel(0.3, Kind_Spatial=2, Kind_Roe=1)
    c.params.precision = abi.TRANS_MIXED
    with pytest.raises(SolverError, match=str(abi.TRANS_E_ARG)):
        Solver(c, conns, geo, st)


RC = dict(Kind_Spatial=3, Kind_Roe=3, Kind_RotMod=1)


def test_rc_correction_channel(gpu_lib):
    """RC correction (Kind_RotMod = 1, Space/RC_Correction.F90:19-124): the rotation/curvature
    factor f_r1 of the SST production (Time/TURBTWO_TIME_LUSGS_SST.F90:286,325), 20 iterations
    bit-identical, with the compressibility correction as well."""
    c, conns, geo, st = small_channel(**RC)
    _run_bitwise(c, conns, geo, st, 20)
    c, conns, geo, st = small_channel(IF_Comppress=1, **RC)
    _run_bitwise(c, conns, geo, st, 10)


def test_rc_correction_cascade(gpu_lib):
    """Five blocks: the face averages and gradients RC reads across block interfaces."""
    from helpers import small_cascade
    c, conns, geo, st = small_cascade(**RC)
    _run_bitwise(c, conns, geo, st, 8)


def test_rc_mode_2_changes_nothing(gpu_lib):
    """Kind_RotMod = 2 computes f_r2 (RC_Correction.F90:126-171), which no routine of the path
    reads: the state is bit-identical to Kind_RotMod = 0."""
    from trans_gb300.solver import Solver
    out = []
    for rot in (0, 2):
        c, conns, geo, st = small_channel(Kind_Spatial=3, Kind_Roe=3, Kind_RotMod=rot)
        s = Solver(c, conns, geo, st)
        for ki in range(1, 6):
            s.iterate(ki)
        out.append(s.get_field(0, "V"))
        s.close()
    assert bit_equal_fraction(out[0], out[1], interior(c.blocks[0].dims)) == 1.0


ROTATING = [dict(Kind_Spatial=3, Kind_Roe=1), dict(Kind_Spatial=2, Kind_Roe=1), dict(Kind_Spatial=1, Kind_Roe=1),
            dict(Kind_Spatial=4, Kind_Roe=1, F_limiter2=0.05), dict(Kind_Spatial=3, Kind_Roe=2),
            dict(Kind_Spatial=3, Kind_Roe=3), dict(Kind_Spatial=3, Kind_Roe=3, Kind_RotMod=1),
            dict(Kind_Spatial=2, Kind_Roe=1, IF_Precondition=1),
            dict(Kind_Spatial=3, Kind_Roe=1, IF_RK=1, CFL_Sub_start=1.0, CFL_Sub_end=1.0)]


@pytest.mark.parametrize("scheme", ROTATING, ids=["mdcd_roe", "muscl_roe", "muscl2_roe", "mdcdhyb_roe", "mdcd_roerot",
                                                  "mdcd_ausmpw", "mdcd_ausmpw_rc", "muscl_roe_precond", "mdcd_roe_rk3"])
def test_rotating_frame(gpu_lib, scheme):
    """A frame rotating about x (omega(1) != 0) on the annular sector, hub turning with the frame
    and casing at rest: the frame speeds rccl/rccr * omega of the Roe schemes (reconstructed as
    each spatial scheme does: limited in MUSCL and MUSCL2, MDCD states in I and J and the face
    average in K for MDCD, the face average for MDCDHYB), the Coriolis and centrifugal source
    of DIFFUSION_Centered.F90:812-822, the rotating wall, inlet and outlet conditions, the
    rothalpy of the update and, with RC correction, omega in the rotation tensor; also with
    low-Mach preconditioning and with the SSP-RK3 stages (whose update has no rotation term, as
    in the reference).  15 iterations bit-identical."""
    from helpers import small_annular
    c, conns, geo, st = small_annular(**scheme)
    assert c.params.omega[0] > 0.5
    _run_bitwise(c, conns, geo, st, 15)


def test_rotating_frame_stage_by_stage(gpu_lib):
    """The residual of the first iteration on its own (MUSCL + Roe): D bit-identical, so a
    missing frame-speed or source term shows up before the update mixes the components."""
    from helpers import small_annular
    c, conns, geo, st = small_annular(Kind_Spatial=2, Kind_Roe=1)
    g, o = _pair(c, conns, geo, st)
    for s in ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL"):
        g.run_stage(s, 1)
        o.run_stage(s, 1)
    m = interior(c.blocks[0].dims)
    a, r = g.get_field(0, "D"), o.get_field(0, "D")
    assert bit_equal_fraction(a, r, m) == 1.0, np.max(rel_err(a, r, m))
    g.close(); o.close()
