"""Caller-side set-up for the TRANS hot path: parameters, connectivity, geometry, initial field.

In the reference these steps stay on the Fortran side (Input/, Geom/); the GPU library receives
their products through the C ABI.  This module restates them so that a case can be driven
without the Fortran code.  Every array is held at the full ghost extent -2..N+2 in each index
direction, in Fortran order, as ``arr[comp..., i+2, j+2, k+2]``; ``fortran_view`` cuts out the
allocation the reference uses for that field.
"""
from dataclasses import dataclass, field
import math

import numpy as np

from . import abi
from . import detmath as dm

G = 2  # index offset of Fortran index 0 (arrays start at -2)


# --------------------------------------------------------------------------------------------
# Parameters (Input/ReadOrg.F90:12-62, Input/ParameterSet.F90:1-96)
# --------------------------------------------------------------------------------------------
@dataclass
class Physical:
    """Dimensional inputs of original.org / dimension_global.dat."""
    XM: float = 0.5
    AoA: float = 0.0
    AoYaw: float = 0.0
    Tinf: float = 288.15
    T0in_K: float = None          # total temperature at the inlet [K]
    P0in_Pa: float = None         # total pressure at the inlet [Pa]
    Pouthub_Pa: float = None      # outlet static pressure at the hub [Pa]
    omega_rpm: tuple = (0.0, 0.0, 0.0)
    FSTI: float = 0.01
    VisRatio: float = 1.0
    nblade: int = 1
    npassage: int = 1


def static_pressure_Pa(Tinf):
    """Static pressure that makes the non-dimensional density 1 (rho_ref = 1.2 kg/m3)."""
    return 1.2 * 287.0 * Tinf


def make_params(ph: Physical, **kw):
    """Module globals after INPUT_ReadOrg, ParameterSet and NonDimensionlization.

    Follows Input/ParameterSet.F90:5-67 and :70-96 operation by operation; keyword arguments
    set the switches of original.org (Input/ReadOrg.F90:13-55).
    """
    p = abi.TransParams()
    # switches with the reference's hard-wired overrides (Input/ReadOrg.F90:59-62)
    sw = dict(Kind_Spatial=2, Kind_Roe=1, F_limiter1=0.0, F_limiter2=0.0, gama_max=0.0463783,
              gama_min=0.0, DT_LUSGS_Main=1.0e8, CFL_Sub_start=5.0, CFL_Sub_end=5.0,
              CFL_Sub_step=1, Kind_Dual=2, Kchld=1, IF_RK=0, IF_Euler=0, IF_Turb_org=1,
              IF_setRkof=0, Rkfset=0.0, Rofset=0.0, KItm=0, Kind_Model=1, Prod_Lmt=20.0,
              IF_Comppress=0, Kind_Hybrid=0, Kind_SubHY=0, If_fix_Transition=0,
              Trans_location=0.0, Alscale=1.0, precision=abi.TRANS_FP64, KI_ini=0,
              IF_Precondition=0, Kind_RotMod=0)
    unknown = set(kw) - set(sw)
    if unknown:
        raise ValueError(f"unknown switches {unknown}")
    sw.update(kw)
    PI = 4 * math.atan(1.0)
    Alfa = ph.AoA / 180.0 * PI
    Beta_Yaw = ph.AoYaw / 180.0 * PI
    p.VxF = dm.cos(Beta_Yaw) * dm.cos(Alfa)
    p.VyF = dm.cos(Beta_Yaw) * dm.sin(Alfa)
    p.VzF = dm.sin(Beta_Yaw)
    gam0 = 1.4
    XM2 = ph.XM * ph.XM
    p.XM = ph.XM
    p.RXM2 = XM2 * gam0
    p.PPF = 1.0 / gam0 / XM2
    p.Csthlnd = 110.0 / ph.Tinf
    p.Csth1 = ph.Tinf / 273.15
    p.Tiny = 1.0e-20                                   # main.F90:12
    if sw["IF_Turb_org"]:
        p.A1, Akapa, p.Beta_star = 0.31, 0.41, 0.09
        if sw["Kind_Model"] == 1:                      # SST (Input/ParameterSet.F90:34-37)
            p.Sigk1, p.Sigo1, p.Beta1, p.Gama1 = 0.85, 0.500, 0.0750, 5.0 / 9.0
            p.Sigk2, p.Sigo2, p.Beta2, p.Gama2 = 1.00, 0.856, 0.0828, 0.440
        elif sw["Kind_Model"] == 2:                    # WD+2006 (Input/ParameterSet.F90:39-43)
            p.Sigk1, p.Sigo1, p.Beta1, p.Gama1 = 0.6, 0.5, 0.0708, 0.52
            p.Sigk2, p.Sigo2, p.Beta2, p.Gama2 = 0.6, 0.5, 0.0708, 0.52
        else:
            raise ValueError("Kind_Model must be 1 (SST) or 2 (WD+2006)")
        p.Rmiuf = 1.8e-5 / 1.2
        p.Rkf = 1.5 * ph.FSTI * ph.FSTI
        p.Rof = 1.2 * p.Rkf / p.Rmiuf
        if sw["IF_setRkof"] == 1:
            p.Rkf, p.Rof = sw["Rkfset"], sw["Rofset"]
    # NonDimensionlization (Input/ParameterSet.F90:70-96)
    T0in = ph.T0in_K / ph.Tinf
    asonic = math.sqrt(1.4 * ph.Tinf * 287)
    Vref = ph.XM * asonic
    Lref = 1.0
    miuref = (1.0 + p.Csthlnd) / (T0in * p.Csth1 + p.Csthlnd) * dm.pow(p.Csth1 * T0in, 1.5) * 1.7e-5
    Roref = 1.2
    p.Ref = Roref * Vref * Lref / miuref
    Pref = Roref * Vref * Vref
    p.P0in = ph.P0in_Pa / Pref
    p.Pouthub = ph.Pouthub_Pa / Pref
    p.T0in = T0in
    for d in range(3):
        p.omega[d] = ph.omega_rpm[d] * 2.0 * PI * Lref / (60.0 * Vref)
    p.VisRatio = ph.VisRatio
    p.FSTI = ph.FSTI
    p.IF_Local_Main, p.IF_Local_Sub, p.CFL_Main = 0, 1, 1.0
    p.DT_LUSGS_Sub = 0.0
    for k in ("Kind_Spatial", "Kind_Roe", "F_limiter1", "F_limiter2", "gama_max", "gama_min",
              "DT_LUSGS_Main", "CFL_Sub_start", "CFL_Sub_end", "CFL_Sub_step", "Kind_Dual",
              "Kchld", "IF_RK", "IF_Euler", "IF_Turb_org", "KItm", "Kind_Model", "Prod_Lmt",
              "IF_Comppress", "Kind_Hybrid", "Kind_SubHY", "If_fix_Transition",
              "Trans_location", "Alscale", "precision", "KI_ini", "IF_Precondition",
              "Kind_RotMod"):
        setattr(p, k, sw[k])
    return p


def params_copy(p):
    q = abi.TransParams()
    C = __import__("ctypes")
    C.memmove(C.addressof(q), C.addressof(p), C.sizeof(p))
    return q


def mu_laminar_nd(p, T):
    """Sutherland viscosity as the hot path evaluates it (Time/SpectralRadius.F90:59)."""
    x = p.Csth1 * T
    return (1.0 + p.Csthlnd) / (T * p.Csth1 + p.Csthlnd) * (x * math.sqrt(x))


# --------------------------------------------------------------------------------------------
# Blocks, BC segments and connectivity (Input/PLOT3DReadInit.F90:19-348)
# --------------------------------------------------------------------------------------------
@dataclass
class Segment:
    """One row of grd/dimension_blkNNN_m.dat (Input/PLOT3DReadInit.F90:38-40)."""
    surf: int                 # 1..6 = imin, imax, jmin, jmax, kmin, kmax
    a0: int = 0               # first/last cell of the first tangential index (0 = full)
    a1: int = 0
    b0: int = 0
    b1: int = 0
    kind: int = 1             # 1 wall, 2 far field, 3 symmetry, 5 inlet, 7 outlet, 9 1-to-1
    kindsub: int = 0
    blk_ex: int = 0           # target block (1-based global id) for kind 9
    blkbd_ex: int = 0         # target segment (1-based) for kind 9
    lcross: int = 0
    lrev_a: int = 0
    lrev_b: int = 0
    period: int = 0


@dataclass
class Block:
    id: int
    xyz: np.ndarray                       # (NI,NJ,NK,3) node coordinates after /alscale
    segments: list
    walls: list = field(default_factory=list)   # (surf, a0, a1, b0, b1) wall-surface entries

    @property
    def dims(self):
        return self.xyz.shape[:3]


@dataclass
class Case:
    name: str
    params: abi.TransParams
    blocks: list
    surfaces: list                        # wall surfaces (Ns,Ms,3) for the wall distance
    physical: Physical = None
    meta: dict = field(default_factory=dict)


def segment_prange(seg, dims):
    """Prange/CPrange of one segment (Input/PLOT3DReadInit.F90:41-117)."""
    NX, NY, NZ = dims
    a0, a1, b0, b1 = seg.a0, seg.a1, seg.b0, seg.b1
    s = seg.surf
    if s in (1, 2):
        a0 = a0 or 1; a1 = a1 or NY - 1; b0 = b0 or 1; b1 = b1 or NZ - 1
        Ib = Ie = (1 if s == 1 else NX)
        Jb, Je, Kb, Ke = a0, a1, b0, b1
    elif s in (3, 4):
        a0 = a0 or 1; a1 = a1 or NX - 1; b0 = b0 or 1; b1 = b1 or NZ - 1
        Jb = Je = (1 if s == 3 else NY)
        Ib, Ie, Kb, Ke = a0, a1, b0, b1
    elif s in (5, 6):
        a0 = a0 or 1; a1 = a1 or NX - 1; b0 = b0 or 1; b1 = b1 or NY - 1
        Kb = Ke = (1 if s == 5 else NZ)
        Ib, Ie, Jb, Je = a0, a1, b0, b1
    else:
        raise ValueError("Wrong Dimension Input!")
    return (Ib, Jb, Kb, Ie, Je, Ke)


def _ftrunc_div(a, b):
    """Fortran integer division (truncation toward zero)."""
    q = abs(a) // abs(b)
    return q if (a >= 0) == (b > 0) else -q


def derive_connectivity(blocks):
    """AConnectivity of every block (Input/PLOT3DReadInit.F90:135-348)."""
    by_id = {b.id: b for b in blocks}
    pr = {b.id: [segment_prange(s, b.dims) for s in b.segments] for b in blocks}
    out = {}
    for b in blocks:
        NDim = b.dims
        conns = []
        for ic, s in enumerate(b.segments):
            c = abi.TransConn()
            c.BCType, c.SubBCType, c.PerType, c.lcross = s.kind, s.kindsub, s.period, s.lcross
            P = pr[b.id][ic]
            for d in range(3):
                c.pointStart[d], c.pointEnd[d] = P[d], P[3 + d]
            c.TargetBlock, c.TargetConn = s.blk_ex, s.blkbd_ex
            c.rotateAngle = 0.0                       # set by set_rotate_angles
            if s.kind == 9 and (s.blk_ex not in by_id or not 1 <= s.blkbd_ex <= len(by_id[s.blk_ex].segments)):
                raise ValueError(f"block {b.id} segment {ic + 1}: bad 1-to-1 target")
            Imin, Jmin, Kmin, Imax, Jmax, Kmax = P
            if Imin == Imax:
                c.IJKDirect = 1
            elif Jmin == Jmax:
                c.IJKDirect = 2
            elif Kmin == Kmax:
                c.IJKDirect = 3
            else:
                raise ValueError("segment is not a face")
            c.LeftOrRight = 1 if ((Imin == Imax and Imin == 1) or (Jmin == Jmax and Jmin == 1)
                                  or (Kmin == Kmax and Kmin == 1)) else 2
            d = c.IJKDirect - 1
            lo = (Imin, Jmin, Kmin)[d]
            for arr in ("IJKAdd", "CIJKAdd", "CIJKAdd1", "CIJKAdd2", "CEIJKAdd", "CEIJKAdd1", "CEIJKAdd2"):
                for q in range(3):
                    getattr(c, arr)[q] = 0
            if lo == 1:
                c.IJKAdd[d], c.CIJKAdd1[d], c.CIJKAdd2[d] = 1, 1, 2
                c.CEIJKAdd1[d], c.CEIJKAdd2[d] = -2, -3
            elif lo == NDim[d]:
                c.IJKAdd[d], c.CIJKAdd1[d], c.CIJKAdd2[d] = -1, -2, -3
                c.CEIJKAdd1[d], c.CEIJKAdd2[d] = 1, 2
            else:
                raise ValueError("face index must be 1 or N")
            for q in range(3):
                c.CIJKAdd[q] = _ftrunc_div(c.IJKAdd[q] - 1, 2)
                c.CEIJKAdd[q] = _ftrunc_div(-c.IJKAdd[q] - 1, 2)
            for q in range(3):
                c.Transform[q] = c.TransformT[q] = c.revMatrix[q] = 0
            c.Transform[d] = 1
            tang = [q for q in range(3) if q != d]
            c.revMatrix[tang[0]] = s.lrev_a
            c.revMatrix[tang[1]] = s.lrev_b
            if s.kind == 9:
                T = pr[s.blk_ex][s.blkbd_ex - 1]
                if T[0] == T[3]:
                    c.TransformT[0] = 1
                elif T[1] == T[4]:
                    c.TransformT[1] = 1
                elif T[2] == T[5]:
                    c.TransformT[2] = 1
            conns.append(c)
        out[b.id] = conns
    return out


def set_rotate_angles(conns, blocks, nblade, npassage):
    """rotateAngle(1) of periodic connections (Input/PLOT3DReadInit.F90:157-160)."""
    PI = 4 * math.atan(1.0)
    for b in blocks:
        for c, s in zip(conns[b.id], b.segments):
            c.rotateAngle = 0.0
            if s.period != 0:
                c.rotateAngle = float(npassage * s.period) * 2 * PI / float(nblade)


def ijk_start_end(i, j, k, TL, TT, lcross):
    """IJKStartEnd (Geom/startup.F90:1-25)."""
    ft1, ft2, ft3 = TL
    gt1, gt2, gt3 = TT
    l1 = 1 - lcross
    t1 = ft1 * i + ft2 * j + ft3 * k
    t2 = ft1 * (j * l1 + k * lcross) + ft2 * (i * l1 + k * lcross) + ft3 * (i * l1 + j * lcross)
    t3 = ft1 * (j * lcross + k * l1) + ft2 * (i * lcross + k * l1) + ft3 * (i * lcross + j * l1)
    Is = gt1 * t1 + (gt2 + gt3) * t2
    Js = gt2 * t1 + gt1 * t2 + gt3 * t3
    Ks = gt3 * t1 + (gt1 + gt2) * t3
    return Is, Js, Ks


def face_cells(c):
    """(i,j,k) arrays of the face cells of a connection, in the reference loop order k,j,i."""
    ks = np.arange(c.pointStart[2], c.pointEnd[2] + 1)
    js = np.arange(c.pointStart[1], c.pointEnd[1] + 1)
    is_ = np.arange(c.pointStart[0], c.pointEnd[0] + 1)
    K, J, I = np.meshgrid(ks, js, is_, indexing="ij")
    return I.ravel(), J.ravel(), K.ravel()


def p2p_source(c, tc, i, j, k):
    """Target-block face cell (ibuf,jbuf,kbuf) for local face cells (BC/BC_P2P.F90:80-85)."""
    Ibgn, Jbgn, Kbgn = c.pointStart
    Iend, Jend, Kend = c.pointEnd
    IIadd, JJadd, KKadd = Iend - Ibgn + 2, Jend - Jbgn + 2, Kend - Kbgn + 2
    iL = i - Ibgn + 1
    jL = j - Jbgn + 1
    kL = k - Kbgn + 1
    rm = c.revMatrix
    iL = rm[0] * IIadd + (1 - 2 * rm[0]) * iL
    jL = rm[1] * JJadd + (1 - 2 * rm[1]) * jL
    kL = rm[2] * KKadd + (1 - 2 * rm[2]) * kL
    Is, Js, Ks = ijk_start_end(iL, jL, kL, tuple(c.Transform), tuple(c.TransformT), c.lcross)
    return Is + tc.pointStart[0] - 1, Js + tc.pointStart[1] - 1, Ks + tc.pointStart[2] - 1


def markwall_arrays(b):
    """MARKWALL* arrays of a block (Input/Read_BlockDimensions.F90:146-283)."""
    NI, NJ, NK = b.dims
    NI1, NJ1, NK1 = NI - 1, NJ - 1, NK - 1
    mw = [np.zeros((NJ1, NK1), np.int32, order="F"), np.zeros((NJ1, NK1), np.int32, order="F"),
          np.zeros((NI1, NK1), np.int32, order="F"), np.zeros((NI1, NK1), np.int32, order="F"),
          np.zeros((NI1, NJ1), np.int32, order="F"), np.zeros((NI1, NJ1), np.int32, order="F")]
    for (surf, a0, a1, b0, b1) in b.walls:
        if surf in (1, 2):
            r = (a0 or 1, a1 or NJ1, b0 or 1, b1 or NK1)
        elif surf in (3, 4):
            r = (a0 or 1, a1 or NI1, b0 or 1, b1 or NK1)
        else:
            r = (a0 or 1, a1 or NI1, b0 or 1, b1 or NJ1)
        mw[surf - 1][r[0] - 1:r[1], r[2] - 1:r[3]] = 1
    return mw


# --------------------------------------------------------------------------------------------
# Geometry (Geom/CalcDst.F90:28-719, Geom/startup.F90:396-755)
# --------------------------------------------------------------------------------------------
def _zeros(ni, nj, nk, comps=()):
    return np.zeros(comps + (ni + 5, nj + 5, nk + 5), dtype=np.float64, order="F")


def wall_distance(xc, yc, zc, surfaces, tiny=1.0e-20):
    """Brute-force nearest panel centre (Geom/CalcDst.F90:127-164), via a k-d tree.

    The tree only finds the nearest panel centre; the squared distance is then evaluated with
    the reference's expression, so the result equals the reference's sequential minimum.
    """
    from scipy.spatial import cKDTree
    pts = np.stack([xc.ravel(), yc.ravel(), zc.ravel()], axis=1)
    dmin = np.full(pts.shape[0], 1.0e20)
    for S in surfaces:
        X, Y, Z = S[..., 0], S[..., 1], S[..., 2]
        xs = (X[:-1, :-1] + X[1:, :-1] + X[:-1, 1:] + X[1:, 1:]) / 4.0
        ys = (Y[:-1, :-1] + Y[1:, :-1] + Y[:-1, 1:] + Y[1:, 1:]) / 4.0
        zs = (Z[:-1, :-1] + Z[1:, :-1] + Z[:-1, 1:] + Z[1:, 1:]) / 4.0
        cen = np.stack([xs.ravel(), ys.ravel(), zs.ravel()], axis=1)
        _, idx = cKDTree(cen).query(pts, k=1)
        dx = pts[:, 0] - cen[idx, 0]
        dy = pts[:, 1] - cen[idx, 1]
        dz = pts[:, 2] - cen[idx, 2]
        d2 = dx * dx + dy * dy + dz * dz
        dmin = np.maximum(dmin, tiny)
        dmin = np.where(d2 < dmin, d2, dmin)
    return np.sqrt(dmin).reshape(xc.shape)


def block_metrics(b, surfaces, tiny=1.0e-20, dst_fn=None, metrics_fn=None):
    """GEOM_CalcDST for one block (Geom/CalcDst.F90:28-719).  dst_fn: the wall-distance
    function (default: `wall_distance` on the host; trans_gb300.solver.device_wall_distance
    evaluates the same minimum on the GPU).  metrics_fn: centres, wall distance, SD/Grad,
    Alagm, boundary face centres, aLeng/aSeng and Vol of the block in one call
    (trans_gb300.solver.device_block_metrics runs them on the GPU; default: the host code
    below); the corner centres and ghost copies follow on the host either way."""
    NI, NJ, NK = b.dims
    g = metrics_fn(b, surfaces, tiny) if metrics_fn is not None else _block_metrics_host(b, surfaces, tiny, dst_fn)
    return _corners_and_ghosts(g, NI, NJ, NK)


def _block_metrics_host(b, surfaces, tiny, dst_fn):
    NI, NJ, NK = b.dims
    NI1, NJ1, NK1 = NI - 1, NJ - 1, NK - 1
    XX, YY, ZZ = (np.asfortranarray(b.xyz[..., q]) for q in range(3))
    g = {n: _zeros(NI, NJ, NK) for n in ("XC", "YC", "ZC", "DST", "ALENG", "ASENG", "VOL", "RAD", "THTC")}
    g["SD"] = _zeros(NI, NJ, NK, (3, 3))
    g["GRAD"] = _zeros(NI, NJ, NK, (3,))
    g["ALAGM"] = _zeros(NI, NJ, NK, (3,))
    Xc, Yc, Zc = g["XC"], g["YC"], g["ZC"]
    # node slices: N(a,b,c) with a in {0,1} meaning I or I+1 for I=1..NI1 (node index I -> array I-1)
    def n8(A, di, dj, dk, ri=NI1, rj=NJ1, rk=NK1, oi=0, oj=0, ok=0):
        return A[oi + di:oi + di + ri, oj + dj:oj + dj + rj, ok + dk:ok + dk + rk]
    ci = slice(G + 1, G + NI)      # cells 1..NI1
    cj = slice(G + 1, G + NJ)
    ck = slice(G + 1, G + NK)
    for A, Cc in ((ZZ, Zc), (YY, Yc), (XX, Xc)):
        s = (n8(A, 1, 1, 1) + n8(A, 1, 1, 0) + n8(A, 1, 0, 1) + n8(A, 1, 0, 0) + n8(A, 0, 1, 1)
             + n8(A, 0, 1, 0) + n8(A, 0, 0, 1) + n8(A, 0, 0, 0))
        Cc[ci, cj, ck] = s / 8.0
    g["THTC"][ci, cj, ck] = dm.atan2(Zc[ci, cj, ck], Yc[ci, cj, ck])
    g["RAD"][ci, cj, ck] = np.sqrt(Yc[ci, cj, ck] * Yc[ci, cj, ck] + Zc[ci, cj, ck] * Zc[ci, cj, ck])
    # wall distance
    g["DST"][ci, cj, ck] = (dst_fn or wall_distance)(Xc[ci, cj, ck], Yc[ci, cj, ck], Zc[ci, cj, ck], surfaces, tiny)
    # SD & Grad
    SD, Gr = g["SD"], g["GRAD"]
    dl = 1.0
    xv = Xc[G + 2, G + 1, G + 1] - Xc[G + 1, G + 1, G + 1]
    yv = Yc[G + 2, G + 1, G + 1] - Yc[G + 1, G + 1, G + 1]
    zv = Zc[G + 2, G + 1, G + 1] - Zc[G + 1, G + 1, G + 1]

    def cross_half(R1, R2):
        R1X, R1Y, R1Z = R1
        R2X, R2Y, R2Z = R2
        return ((R1Y * R2Z - R1Z * R2Y) * 0.5, (R1Z * R2X - R1X * R2Z) * 0.5, (R1X * R2Y - R1Y * R2X) * 0.5)

    # I faces: I=1..NI, J=1..NJ1, K=1..NK1
    def nd(A, i0, i1, j0, j1, k0, k1):
        return A[i0 - 1:i1, j0 - 1:j1, k0 - 1:k1]
    R1 = [nd(A, 1, NI, 2, NJ, 2, NK) - nd(A, 1, NI, 1, NJ1, 1, NK1) for A in (XX, YY, ZZ)]
    R2 = [nd(A, 1, NI, 1, NJ1, 2, NK) - nd(A, 1, NI, 2, NJ, 1, NK1) for A in (XX, YY, ZZ)]
    xs = cross_half(R1, R2)
    if xv * xs[0][0, 0, 0] + yv * xs[1][0, 0, 0] + zv * xs[2][0, 0, 0] < 0:
        dl = -1.0
    fi, fj, fk = slice(G + 1, G + NI + 1), slice(G + 1, G + NJ), slice(G + 1, G + NK)
    for c in range(3):
        SD[0, c, fi, fj, fk] = xs[c] * dl
    Gr[0, fi, fj, fk] = np.sqrt(SD[0, 0, fi, fj, fk] * SD[0, 0, fi, fj, fk] + SD[0, 1, fi, fj, fk] * SD[0, 1, fi, fj, fk]
                                + SD[0, 2, fi, fj, fk] * SD[0, 2, fi, fj, fk] + tiny)
    SD[0, :, G, fj, fk] = SD[0, :, G + 1, fj, fk]
    Gr[0, G, fj, fk] = Gr[0, G + 1, fj, fk]
    # J faces: K=1..NK1, I=1..NI1, J=1..NJ
    R1 = [nd(A, 1, NI1, 1, NJ, 2, NK) - nd(A, 2, NI, 1, NJ, 1, NK1) for A in (XX, YY, ZZ)]
    R2 = [nd(A, 2, NI, 1, NJ, 2, NK) - nd(A, 1, NI1, 1, NJ, 1, NK1) for A in (XX, YY, ZZ)]
    xs = cross_half(R1, R2)
    fi, fj, fk = slice(G + 1, G + NI), slice(G + 1, G + NJ + 1), slice(G + 1, G + NK)
    for c in range(3):
        SD[1, c, fi, fj, fk] = xs[c] * dl
    Gr[1, fi, fj, fk] = np.sqrt(SD[1, 0, fi, fj, fk] * SD[1, 0, fi, fj, fk] + SD[1, 1, fi, fj, fk] * SD[1, 1, fi, fj, fk]
                                + SD[1, 2, fi, fj, fk] * SD[1, 2, fi, fj, fk] + tiny)
    SD[1, :, fi, G, fk] = SD[1, :, fi, G + 1, fk]
    Gr[1, fi, G, fk] = Gr[1, fi, G + 1, fk]
    # K faces: J=1..NJ1, I=1..NI1, K=1..NK
    R1 = [nd(A, 2, NI, 1, NJ1, 1, NK) - nd(A, 1, NI1, 2, NJ, 1, NK) for A in (XX, YY, ZZ)]
    R2 = [nd(A, 2, NI, 2, NJ, 1, NK) - nd(A, 1, NI1, 1, NJ1, 1, NK) for A in (XX, YY, ZZ)]
    xs = cross_half(R1, R2)
    fi, fj, fk = slice(G + 1, G + NI), slice(G + 1, G + NJ), slice(G + 1, G + NK + 1)
    for c in range(3):
        SD[2, c, fi, fj, fk] = xs[c] * dl
    Gr[2, fi, fj, fk] = np.sqrt(SD[2, 0, fi, fj, fk] * SD[2, 0, fi, fj, fk] + SD[2, 1, fi, fj, fk] * SD[2, 1, fi, fj, fk]
                                + SD[2, 2, fi, fj, fk] * SD[2, 2, fi, fj, fk] + tiny)
    SD[2, :, fi, fj, G] = SD[2, :, fi, fj, G + 1]
    Gr[2, fi, fj, G] = Gr[2, fi, fj, G + 1]
    # Alagm (Geom/CalcDst.F90:322-358)
    Al = g["ALAGM"]
    def q4(A, a, b, c, d):
        return 0.25 * (a(A) + b(A) + c(A) + d(A))
    def N(di, dj, dk):
        return lambda A: A[di:di + NI1, dj:dj + NJ1, dk:dk + NK1]
    fc = {}
    for nm, A in (("x", XX), ("y", YY), ("z", ZZ)):
        fc["w" + nm] = q4(A, N(0, 0, 0), N(0, 1, 0), N(0, 0, 1), N(0, 1, 1))
        fc["e" + nm] = q4(A, N(1, 0, 0), N(1, 1, 0), N(1, 0, 1), N(1, 1, 1))
        fc["s" + nm] = q4(A, N(0, 0, 0), N(1, 0, 0), N(0, 0, 1), N(1, 0, 1))
        fc["n" + nm] = q4(A, N(0, 1, 0), N(1, 1, 0), N(0, 1, 1), N(1, 1, 1))
        fc["b" + nm] = q4(A, N(0, 0, 0), N(1, 0, 0), N(0, 1, 0), N(1, 1, 0))
        fc["t" + nm] = q4(A, N(0, 0, 1), N(1, 0, 1), N(0, 1, 1), N(1, 1, 1))
    for d, (a, bb) in enumerate((("w", "e"), ("s", "n"), ("b", "t"))):
        dx = fc[a + "x"] - fc[bb + "x"]
        dy = fc[a + "y"] - fc[bb + "y"]
        dz = fc[a + "z"] - fc[bb + "z"]
        Al[d, ci, cj, ck] = np.sqrt(dx * dx + dy * dy + dz * dz)
    # boundary face centres (Geom/CalcDst.F90:370-422)
    for A, Cc in ((XX, Xc), (YY, Yc), (ZZ, Zc)):
        for ii, gi in ((1, G + 0), (NI, G + NI)):
            Cc[gi, cj, ck] = (A[ii - 1, 0:NJ1, 0:NK1] + A[ii - 1, 1:NJ, 0:NK1] + A[ii - 1, 0:NJ1, 1:NK]
                              + A[ii - 1, 1:NJ, 1:NK]) / 4.0
        for jj, gj in ((1, G + 0), (NJ, G + NJ)):
            Cc[ci, gj, ck] = (A[0:NI1, jj - 1, 0:NK1] + A[1:NI, jj - 1, 0:NK1] + A[0:NI1, jj - 1, 1:NK]
                              + A[1:NI, jj - 1, 1:NK]) / 4.0
        for kk, gk in ((1, G + 0), (NK, G + NK)):
            Cc[ci, cj, gk] = (A[0:NI1, 0:NJ1, kk - 1] + A[1:NI, 0:NJ1, kk - 1] + A[0:NI1, 1:NJ, kk - 1]
                              + A[1:NI, 1:NJ, kk - 1]) / 4.0
    # aLeng / aSeng (Geom/CalcDst.F90:430-480)
    c0 = (ci, cj, ck)
    def sh(A, di, dj, dk):
        return A[G + 1 + di:G + NI + di, G + 1 + dj:G + NJ + dj, G + 1 + dk:G + NK + dk]
    dd = []
    for (di, dj, dk) in ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)):
        dx = sh(Xc, di, dj, dk) - Xc[c0]
        dy = sh(Yc, di, dj, dk) - Yc[c0]
        dz = sh(Zc, di, dj, dk) - Zc[c0]
        dd.append(np.sqrt(dx * dx + dy * dy + dz * dz))
    DDw, DDe, DDs, DDn, DDl, DDu = dd
    DLT = np.maximum.reduce(dd)
    DST = np.minimum.reduce(dd)
    if NI1 == 2:
        DLT = np.maximum.reduce([DDs, DDn, DDl, DDu])
    if NJ1 == 2:
        DLT = np.maximum.reduce([DDw, DDe, DDl, DDu])
    if NK1 == 2:
        DLT = np.maximum.reduce([DDw, DDe, DDs, DDn])
    if NI1 == 2:
        DST = np.minimum.reduce([DDs, DDn, DDl, DDu])
    if NJ1 == 2:
        DST = np.minimum.reduce([DDw, DDe, DDl, DDu])
    if NK1 == 2:
        DST = np.minimum.reduce([DDw, DDe, DDs, DDn])
    g["ALENG"][c0] = DLT
    g["ASENG"][c0] = DST
    # Vol (Geom/CalcDst.F90:488-521)
    C13 = 1.0 / 3.0
    def nn(A, di, dj, dk):
        return A[di:di + NI1, dj:dj + NJ1, dk:dk + NK1]
    sd = lambda d, c: SD[d, c, ci, cj, ck]
    XR = nn(XX, 1, 1, 1) - nn(XX, 0, 1, 1); YR = nn(YY, 1, 1, 1) - nn(YY, 0, 1, 1); ZR = nn(ZZ, 1, 1, 1) - nn(ZZ, 0, 1, 1)
    OMG = XR * sd(0, 0) + YR * sd(0, 1) + ZR * sd(0, 2)
    XR = nn(XX, 1, 1, 1) - nn(XX, 1, 0, 1); YR = nn(YY, 1, 1, 1) - nn(YY, 1, 0, 1); ZR = nn(ZZ, 1, 1, 1) - nn(ZZ, 1, 0, 1)
    OMG = OMG + XR * sd(1, 0) + YR * sd(1, 1) + ZR * sd(1, 2)
    XR = nn(XX, 1, 1, 1) - nn(XX, 1, 1, 0); YR = nn(YY, 1, 1, 1) - nn(YY, 1, 1, 0); ZR = nn(ZZ, 1, 1, 1) - nn(ZZ, 1, 1, 0)
    OMG = OMG + XR * sd(2, 0) + YR * sd(2, 1) + ZR * sd(2, 2)
    g["VOL"][c0] = C13 * OMG
    if np.any(g["VOL"][c0] < tiny):
        raise ValueError(f"block {b.id}: negative volume")
    return g


def _corners_and_ghosts(g, NI, NJ, NK):
    NI1, NJ1, NK1 = NI - 1, NJ - 1, NK - 1
    ci, cj, ck = slice(G + 1, G + NI), slice(G + 1, G + NJ), slice(G + 1, G + NK)
    Xc, Yc, Zc, SD, Al = g["XC"], g["YC"], g["ZC"], g["SD"], g["ALAGM"]
    # corner centres (Geom/CalcDst.F90:530-581)
    for Cc in (Xc, Yc, Zc):
        for j in range(1, NJ1 + 1):
            for (ii, kk, k1, k2) in ((0, 0, 1, 2), (0, NK, NK1, NK1 - 1), (NI, 0, 1, 2), (NI, NK, NK1, NK1 - 1)):
                Cc[G + ii, G + j, G + kk] = 1.5 * Cc[G + ii, G + j, G + k1] - Cc[G + ii, G + j, G + k2] * 0.5
        for k in range(0, NK + 1):
            for (ii, jj, j1, j2) in ((0, 0, 1, 2), (0, NJ, NJ1, NJ1 - 1), (NI, 0, 1, 2), (NI, NJ, NJ1, NJ1 - 1)):
                Cc[G + ii, G + jj, G + k] = 1.5 * Cc[G + ii, G + j1, G + k] - Cc[G + ii, G + j2, G + k] * 0.5
        for i in range(0, NI + 1):
            for (jj, kk, j1, j2) in ((0, 0, 1, 2), (NJ, 0, NJ1, NJ1 - 1), (0, NK, 1, 2), (NJ, NK, NJ1, NJ1 - 1)):
                Cc[G + i, G + jj, G + kk] = 1.5 * Cc[G + i, G + j1, G + kk] - Cc[G + i, G + j2, G + kk] * 0.5
    # ghost copies (Geom/CalcDst.F90:585-640)
    V, D_ = g["VOL"], g["DST"]
    for A in (V, D_):
        A[G + 0, cj, ck] = A[G + 1, cj, ck]; A[G + NI, cj, ck] = A[G + NI1, cj, ck]
    Al[0, G + 0, cj, ck] = Al[0, G + 1, cj, ck]; Al[0, G + NI, cj, ck] = Al[0, G + NI1, cj, ck]
    for A in (V, D_):
        A[ci, G + 0, ck] = A[ci, G + 1, ck]; A[ci, G + NJ, ck] = A[ci, G + NJ1, ck]
    Al[1, ci, G + 0, ck] = Al[1, ci, G + 1, ck]; Al[1, ci, G + NJ, ck] = Al[1, ci, G + NJ1, ck]
    for A in (V, D_):
        A[ci, cj, G + 0] = A[ci, cj, G + 1]; A[ci, cj, G + NK] = A[ci, cj, G + NK1]
    Al[2, ci, cj, G + 0] = Al[2, ci, cj, G + 1]; Al[2, ci, cj, G + NK] = Al[2, ci, cj, G + NK1]
    aj, ak = slice(G + 1, G + NJ + 1), slice(G + 1, G + NK + 1)
    ai = slice(G + 1, G + NI + 1)
    SD[0, :, G + 0, aj, ak] = SD[0, :, G + 2, aj, ak]
    SD[0, :, G + NI + 1, aj, ak] = SD[0, :, G + NI1, aj, ak]
    SD[1, :, ai, G + 0, ak] = SD[1, :, ai, G + 2, ak]
    SD[1, :, ai, G + NJ + 1, ak] = SD[1, :, ai, G + NJ1, ak]
    SD[2, :, ai, aj, G + 0] = SD[2, :, ai, aj, G + 2]
    SD[2, :, ai, aj, G + NK + 1] = SD[2, :, ai, aj, G + NK1]
    return g


def _idx(i, j, k):
    return (np.asarray(i) + G, np.asarray(j) + G, np.asarray(k) + G)


def geom_transform(blocks, conns, geo):
    """Ghost metrics at physical boundaries (Geom/startup.F90:396-508)."""
    for b in blocks:
        g = geo[b.id]
        Vol, Dst, Al, rad, th, SD = g["VOL"], g["DST"], g["ALAGM"], g["RAD"], g["THTC"], g["SD"]
        for c in conns[b.id]:
            if c.BCType == 9:
                continue
            i, j, k = face_cells(c)
            d = c.IJKDirect - 1
            s0 = _idx(i + c.CIJKAdd[0], j + c.CIJKAdd[1], k + c.CIJKAdd[2])
            s1 = _idx(i + c.CIJKAdd1[0], j + c.CIJKAdd1[1], k + c.CIJKAdd1[2])
            l0 = _idx(i + c.CEIJKAdd[0], j + c.CEIJKAdd[1], k + c.CEIJKAdd[2])
            l1 = _idx(i + c.CEIJKAdd1[0], j + c.CEIJKAdd1[1], k + c.CEIJKAdd1[2])
            l2 = _idx(i + c.CEIJKAdd2[0], j + c.CEIJKAdd2[1], k + c.CEIJKAdd2[2])
            for A in (Vol, Dst):
                A[l0] = A[s0]
            Al[(d,) + l0] = Al[(d,) + s0]
            for A in (Vol, Dst):
                A[l1] = A[s0]
                A[l2] = A[s0]
            Al[(d,) + l1] = Al[(d,) + s0]
            Al[(d,) + l2] = Al[(d,) + s0]
            for A in (rad, th):
                A[l0] = 2.0 * A[s0] - A[s1]
                A[l1] = 2.0 * A[l0] - A[s0]
                A[l2] = 2.0 * A[l1] - A[l0]
            if c.BCType == 5:
                for A in (rad, th):
                    A[l0] = A[s0]; A[l1] = A[s0]; A[l2] = A[s0]
            sf = _idx(i + c.IJKAdd[0], j + c.IJKAdd[1], k + c.IJKAdd[2])
            lf = _idx(i - c.IJKAdd[0], j - c.IJKAdd[1], k - c.IJKAdd[2])
            f0 = _idx(i, j, k)
            for q in range(3):
                SD[(d, q) + lf] = 2.0 * SD[(d, q) + f0] - SD[(d, q) + sf]


def geom_transform1(blocks, conns, geo):
    """Ghost metrics at 1-to-1 interfaces (Geom/startup.F90:510-755), without MPI."""
    by_id = {b.id: b for b in blocks}
    # pack (send side): for each connection, 18 words per face cell in buffer coordinates
    bufs = {}
    for b in blocks:
        g = geo[b.id]
        for ic, c in enumerate(conns[b.id]):
            if c.BCType != 9:
                continue
            i, j, k = face_cells(c)
            d = c.IJKDirect - 1
            s = [_idx(i + a[0], j + a[1], k + a[2]) for a in (c.CIJKAdd, c.CIJKAdd1, c.CIJKAdd2)]
            ni = c.pointEnd[0] - c.pointStart[0] + 1
            nj = c.pointEnd[1] - c.pointStart[1] + 1
            nk = c.pointEnd[2] - c.pointStart[2] + 1
            buf = np.zeros((18, ni, nj, nk), order="F")
            bi, bj, bk = i - c.pointStart[0], j - c.pointStart[1], k - c.pointStart[2]
            for q, A in enumerate((g["VOL"], g["DST"])):
                for L in range(3):
                    buf[3 * q + L, bi, bj, bk] = A[s[L]]
            for L in range(3):
                buf[6 + L, bi, bj, bk] = g["ALAGM"][(d,) + s[L]]
                buf[9 + L, bi, bj, bk] = g["RAD"][s[L]]
                buf[12 + L, bi, bj, bk] = g["THTC"][s[L]]
            sf = _idx(i + c.IJKAdd[0], j + c.IJKAdd[1], k + c.IJKAdd[2])
            out_n = float(2 * c.LeftOrRight - 3)
            for q in range(3):
                buf[15 + q, bi, bj, bk] = g["SD"][(d, q) + sf] * out_n
            # tag = target block/conn: the receiver of this buffer is (TargetBlock, TargetConn)
            bufs[(c.TargetBlock, c.TargetConn)] = buf
    # unpack (receive side)
    for b in blocks:
        g = geo[b.id]
        for ic, c in enumerate(conns[b.id]):
            if c.BCType != 9:
                continue
            buf = bufs[(b.id, ic + 1)]
            i, j, k = face_cells(c)
            d = c.IJKDirect - 1
            dcita = c.rotateAngle
            sint, cost = dm.sin(dcita), dm.cos(dcita)
            Ibgn, Jbgn, Kbgn = c.pointStart
            Iend, Jend, Kend = c.pointEnd
            IIadd, JJadd, KKadd = Iend - Ibgn + 2, Jend - Jbgn + 2, Kend - Kbgn + 2
            iL, jL, kL = i - Ibgn + 1, j - Jbgn + 1, k - Kbgn + 1
            rm = c.revMatrix
            iL = rm[0] * IIadd + (1 - 2 * rm[0]) * iL
            jL = rm[1] * JJadd + (1 - 2 * rm[1]) * jL
            kL = rm[2] * KKadd + (1 - 2 * rm[2]) * kL
            Is, Js, Ks = ijk_start_end(iL, jL, kL, tuple(c.Transform), tuple(c.TransformT), c.lcross)
            bi, bj, bk = Is - 1, Js - 1, Ks - 1
            l = [_idx(i + a[0], j + a[1], k + a[2]) for a in (c.CEIJKAdd, c.CEIJKAdd1, c.CEIJKAdd2)]
            for q, A in enumerate((g["VOL"], g["DST"])):
                for L in range(3):
                    A[l[L]] = buf[3 * q + L, bi, bj, bk]
            for L in range(3):
                g["ALAGM"][(d,) + l[L]] = buf[6 + L, bi, bj, bk]
                g["RAD"][l[L]] = buf[9 + L, bi, bj, bk]
                g["THTC"][l[L]] = buf[12 + L, bi, bj, bk] - dcita
            if c.PerType != 0:
                s1 = _idx(i + c.CIJKAdd[0], j + c.CIJKAdd[1], k + c.CIJKAdd[2])
                s2 = _idx(i + c.CIJKAdd1[0], j + c.CIJKAdd2[1], k + c.CIJKAdd1[2])
                for A in (g["THTC"], g["RAD"]):
                    A[l[0]] = 2.0 * A[s1] - A[s2]
                    A[l[1]] = 2.0 * A[l[0]] - A[s1]
                    A[l[2]] = 2.0 * A[l[1]] - A[l[0]]
            lf = _idx(i - c.IJKAdd[0], j - c.IJKAdd[1], k - c.IJKAdd[2])
            out_n = float(2 * c.LeftOrRight - 3)
            SD = g["SD"]
            SD[(d, 0) + lf] = -out_n * buf[15, bi, bj, bk]
            SDy = -out_n * buf[16, bi, bj, bk]
            SDz = -out_n * buf[17, bi, bj, bk]
            SD[(d, 1) + lf] = cost * SDy + sint * SDz
            SD[(d, 2) + lf] = -sint * SDy + cost * SDz
            if c.PerType != 0:
                sf = _idx(i + c.IJKAdd[0], j + c.IJKAdd[1], k + c.IJKAdd[2])
                f0 = _idx(i, j, k)
                for q in range(3):
                    SD[(d, q) + lf] = 2.0 * SD[(d, q) + f0] - SD[(d, q) + sf]


def compute_geometry(case, dst_fn=None, metrics_fn=None):
    """All metrics of a case: CalcDst per block, then GeomTransform and GeomTransform1.
    dst_fn, metrics_fn: see block_metrics."""
    conns = derive_connectivity(case.blocks)
    ph = case.physical
    set_rotate_angles(conns, case.blocks, ph.nblade if ph else 1, ph.npassage if ph else 1)
    geo = {b.id: block_metrics(b, case.surfaces, case.params.Tiny, dst_fn, metrics_fn) for b in case.blocks}
    geom_transform(case.blocks, conns, geo)
    geom_transform1(case.blocks, conns, geo)
    return conns, geo


# --------------------------------------------------------------------------------------------
# Initial field (Input/Init.F90:94-169) and the seeded restart perturbation
# --------------------------------------------------------------------------------------------
def standard_normal(rng, shape):
    """N(0,1) draws by the Box-Muller transform of the generator's uniform doubles, with the
    platform-independent log/sin/cos of detmath (numpy's own normal sampler calls libm)."""
    n = int(np.prod(shape))
    m = (n + 1) // 2
    u1 = 1.0 - rng.random(m)                  # (0, 1]
    u2 = rng.random(m)
    r = np.sqrt(-2.0 * dm.log(u1))
    t = 2.0 * dm.pi * u2
    z = np.concatenate([r * dm.cos(t), r * dm.sin(t)])[:n]
    return z.reshape(shape)


def initial_state(case, geo, Q_dst=0.01, If_NS_uniform=0, noise=1.0e-4, seed=0, velocity_noise=None):
    """The reference's KR=0 initialisation (Input/Init.F90:94-169) plus seeded perturbations:
    `noise` relative Gaussian on the density (drawn from `seed`) and, if the case asks for it
    (meta "velocity_noise"), a relative Gaussian perturbation of the streamwise velocity drawn
    from seed+1 (the density stream is unchanged by it)."""
    if velocity_noise is None:
        velocity_noise = case.meta.get("velocity_noise", 0.0)
    vrng = np.random.default_rng(seed + 1)
    p = case.params
    rng = np.random.default_rng(seed)
    st = {}
    for b in case.blocks:
        NI, NJ, NK = b.dims
        g = geo[b.id]
        V = _zeros(NI, NJ, NK, (7,))
        PP, T, Rmiu = _zeros(NI, NJ, NK), _zeros(NI, NJ, NK), _zeros(NI, NJ, NK)
        c0 = (slice(G + 1, G + NI), slice(G + 1, G + NJ), slice(G + 1, G + NK))
        Dst, Yc, Zc, rad = g["DST"][c0], g["YC"][c0], g["ZC"][c0], g["RAD"][c0]
        om = p.omega[0]
        Coff_dst = 4.6 / Q_dst
        V1 = np.ones_like(Dst)
        V2 = np.ones_like(Dst)
        V3 = om * Zc
        V4 = -om * Yc
        ptemp = 1.0 / (1.4 * p.XM * p.XM)
        P = np.full_like(Dst, ptemp)
        if If_NS_uniform == 0:
            Rat = 1.0 - dm.exp(-Coff_dst * Dst)
            V2 = np.where(Dst < Q_dst, V2 * Rat, V2)
        if velocity_noise:
            V2 = V2 * (1.0 + velocity_noise * standard_normal(vrng, Dst.shape))
        V5 = P / 0.4 + 0.5 * (V2 * V2 + V3 * V3 + V4 * V4) - 0.5 * ((om * rad) * (om * rad))
        C1, C2 = 45.8, 1.68
        Smax = C2 / (2.0 * C1)
        tmax = -C1 * Smax * Smax + C2 * Smax
        aKin = np.maximum(p.Rkf, -(C1 * (Dst * Dst)) + C2 * Dst)
        v3d = 100.0 * aKin / tmax
        aOin = np.maximum(-12444.0 * Dst + 0.54, aKin / v3d)
        V[0][c0], V[1][c0], V[2][c0], V[3][c0], V[4][c0] = V1, V2, V3, V4, V5
        V[5][c0], V[6][c0] = aKin, aOin
        Rmiu[c0] = p.Rmiuf
        # seeded restart perturbation of the density
        if noise:
            V[0][c0] = V[0][c0] * (1.0 + noise * standard_normal(rng, Dst.shape))
        Wt0 = V.copy(order="F")
        Wt1 = V.copy(order="F")
        # PP and T from V (Input/Init.F90:156-169)
        VV = V[1][c0] * V[1][c0] + V[2][c0] * V[2][c0] + V[3][c0] * V[3][c0]
        PP[c0] = (1.4 - 1.0) * V[4][c0] - 0.5 * (1.4 - 1.0) * (VV / V[0][c0] + -((om * rad) * (om * rad)) * V[0][c0])
        T[c0] = p.RXM2 * PP[c0] / V[0][c0]
        st[b.id] = dict(V=V, PP=PP, T=T, RMIU=Rmiu, WT0=Wt0, WT1=Wt1)
    return st


def fortran_view(name, arr):
    """Cut the reference allocation of field `name` out of a full-extent (-2..N+2) array."""
    comps, lb = abi.FIELD_LAYOUT[name]
    o = lb + G
    sl = (slice(None),) * len(comps) + (slice(o, None),) * 3
    return np.asfortranarray(arr[sl])


def full_from_fortran(name, farr, ni, nj, nk):
    comps, lb = abi.FIELD_LAYOUT[name]
    full = _zeros(ni, nj, nk, comps)
    o = lb + G
    full[(slice(None),) * len(comps) + (slice(o, None),) * 3] = farr
    return full
