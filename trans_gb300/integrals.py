"""Integrated quantities of a solution, for the precision error table and for retirement
decisions: mass flow through every inlet and outlet, mass-averaged total pressure and the
total-pressure loss coefficient, blade loading (pressure coefficient on the blade wall),
pressure and viscous force on the walls, and field L-inf differences.

Semantics follow the reference's output routines, generalised to every inlet/outlet face:
  mass flow       Output/OUTPUT_Residual_NS.F90:37-75 (face momentum from the two cells'
                  volume-weighted average, dotted with SD of the face; nondimensional units)
  pressure coeff. Output/OUTPUT_Surfaces.F90:303-305 (Cp = 2 (p - PPF) at the wall cell)
  total pressure  Output/Average_Field.F90:66,157 (p (1 + 0.2 M^2)^3.5, mass averaged)
  wall force      Output/OUTPUT_ClCdCm.F90:114-264 (pressure part (p - PPF) S Sgn, viscous part
                  mu_w/(Dst Ref) times the tangential velocity times |S|; before 2/Area_Ref)
  wall moment     Output/OUTPUT_ClCdCm.F90:250-265 (face force times the arm from the reference
                  point to the face centre, the mean of the face's four nodes)
This is a host (numpy) evaluation from downloaded fields; the library computes the same sums
on the device (trans_get_integrals), and the tests hold the two against each other.
Inputs are the full-extent (-2..N+2) arrays of trans_gb300.solver / oracle get_field.
"""
import numpy as np

from .case import G, face_cells

GAM = 1.4


def _face_pairs(cn):
    """Interior cell and ghost cell (Fortran indices) on both sides of each face of a
    boundary connection, and the face index at which SD of the face is stored."""
    I, J, K = face_cells(cn)
    d = cn.IJKDirect - 1
    n = [I.copy(), J.copy(), K.copy()]
    inner = [I.copy(), J.copy(), K.copy()]
    ghost = [I.copy(), J.copy(), K.copy()]
    face = [I.copy(), J.copy(), K.copy()]
    if cn.pointStart[d] == 1:            # min face: face 1 between ghost 0 and cell 1
        ghost[d] = n[d] - 1
        face[d] = n[d]
    else:                                 # max face N: between cell N-1 and ghost N
        inner[d] = n[d] - 1
        face[d] = n[d]
    return d, tuple(inner), tuple(ghost), tuple(face), cn.pointStart[d] == 1


def _at(a, ijk, comp=()):
    i, j, k = ijk
    comp = comp if isinstance(comp, tuple) else (comp,)
    return a[comp + (i + G, j + G, k + G)]


def boundary_flux(case, conns, geo, fields, kind):
    """Mass flow and mass-averaged total pressure and static pressure through every face of
    the given BC kind.  Returns (mass, p0_mass_avg, p_mass_avg); mass > 0 into the domain for
    inflow faces (kind 5) and out of it for outflow faces (kind 7)."""
    m_tot, p0m, pm = 0.0, 0.0, 0.0
    for ib, b in enumerate(case.blocks):
        g = geo[b.id]
        V, PP = fields[ib]["V"], fields[ib]["PP"]
        vol = g["VOL"]
        for cn in conns[b.id]:
            if cn.BCType != kind:
                continue
            d, ci, cg, cf, is_min = _face_pairs(cn)
            w1 = _at(vol, cg)             # weights crossed as in the reference
            w2 = _at(vol, ci)
            wsum = w1 + w2
            ru = [(w1 * _at(V, ci, q) + w2 * _at(V, cg, q)) / wsum for q in (1, 2, 3)]
            rho = (w1 * _at(V, ci, 0) + w2 * _at(V, cg, 0)) / wsum
            p = (w1 * _at(PP, ci) + w2 * _at(PP, cg)) / wsum
            S = [_at(g["SD"], cf, (d, q)) for q in range(3)]
            flux = ru[0] * S[0] + ru[1] * S[1] + ru[2] * S[2]      # along +IJKDirect
            into = (kind == 5) == is_min      # inflow through a min face, outflow through a max face
            mf = flux if into else -flux
            u2 = (ru[0] ** 2 + ru[1] ** 2 + ru[2] ** 2) / (rho * rho)
            M2 = u2 / (GAM * p / rho)
            p0 = p * (1.0 + 0.5 * (GAM - 1.0) * M2) ** (GAM / (GAM - 1.0))
            m_tot += float(np.sum(mf))
            p0m += float(np.sum(mf * p0))
            pm += float(np.sum(mf * p))
    if m_tot == 0.0:
        return 0.0, 0.0, 0.0
    return m_tot, p0m / m_tot, pm / m_tot


def loss_coefficient(case, conns, geo, fields):
    """Total-pressure loss (P0in - P0out) / (P0in - pin), mass averaged over inlet/outlet."""
    _, p0i, pi = boundary_flux(case, conns, geo, fields, 5)
    _, p0o, _ = boundary_flux(case, conns, geo, fields, 7)
    return (p0i - p0o) / (p0i - pi)


def wall_cp(case, conns, geo, fields, block_index=0, surf_dir=2, k_index=None):
    """Pressure coefficient 2 (p - PPF) on the wall cells of the j-min face of one block
    (the blade of the cascade O-block) at span station k_index (default mid-span)."""
    b = case.blocks[block_index]
    ni, nj, nk = b.dims
    k = (nk - 1) // 2 + 1 if k_index is None else k_index
    PP = fields[block_index]["PP"]
    p = PP[G + 1:G + ni, G + 1, G + k]
    return 2.0 * (p - case.params.PPF)


def wall_forces(case, conns, geo, fields):
    """Pressure and viscous force summed over every wall face (kind 1), nondimensional, before
    the reference's 2/Area_Ref scaling (Output/OUTPUT_ClCdCm.F90:199-248)."""
    P = case.params
    Fp, Fv = np.zeros(3), np.zeros(3)
    for ib, b in enumerate(case.blocks):
        g = geo[b.id]
        V, PP, T = fields[ib]["V"], fields[ib]["PP"], fields[ib]["T"]
        for cn in conns[b.id]:
            if cn.BCType != 1:
                continue
            d, ci, cg, cf, is_min = _face_pairs(cn)
            Sl = _at(g["GRAD"], cf, d)
            S = [_at(g["SD"], cf, (d, q)) / Sl for q in range(3)]
            sgn = -1.0 if is_min else 1.0
            P2 = _at(PP, ci) - P.PPF
            for q in range(3):
                Fp[q] += float(np.sum(P2 * S[q] * Sl * sgn))
            TT = _at(T, ci)
            mu_w = (1.0 + P.Csthlnd) / (TT * P.Csth1 + P.Csthlnd) * (P.Csth1 * TT) ** 1.5
            den = _at(V, ci, 0)
            u = [_at(V, ci, q + 1) / den for q in range(3)]
            vcon = u[0] * S[0] * Sl + u[1] * S[1] * Sl + u[2] * S[2] * Sl
            tau = 1.0 * mu_w / _at(geo[b.id]["DST"], ci) / P.Ref
            for q in range(3):
                Fv[q] += float(np.sum(tau * (u[q] * Sl - vcon * S[q])))
    return Fp, Fv


def segment_wall_forces(case, conns, geo, fields, ib, iconn):
    """Pressure and viscous force of each face of wall segment iconn (1-based) of block ib, as
    an array (6, nfaces): rows pressure x, y, z, viscous x, y, z; the faces I fastest, then J,
    then K (the per-face terms of wall_forces, Output/OUTPUT_ClCdCm.F90:199-248)."""
    P = case.params
    b = case.blocks[ib]
    g = geo[b.id]
    cn = conns[b.id][iconn - 1]
    V, PP, T = fields[ib]["V"], fields[ib]["PP"], fields[ib]["T"]
    d, ci, cg, cf, is_min = _face_pairs(cn)
    Sl = _at(g["GRAD"], cf, d)
    S = [_at(g["SD"], cf, (d, q)) / Sl for q in range(3)]
    sgn = -1.0 if is_min else 1.0
    P2 = _at(PP, ci) - P.PPF
    TT = _at(T, ci)
    mu_w = (1.0 + P.Csthlnd) / (TT * P.Csth1 + P.Csthlnd) * (P.Csth1 * TT) ** 1.5
    den = _at(V, ci, 0)
    u = [_at(V, ci, q + 1) / den for q in range(3)]
    vcon = u[0] * S[0] * Sl + u[1] * S[1] * Sl + u[2] * S[2] * Sl
    tau = 1.0 * mu_w / _at(g["DST"], ci) / P.Ref
    out = np.empty((6, len(P2)))
    for q in range(3):
        out[q] = P2 * S[q] * Sl * sgn
        out[3 + q] = tau * (u[q] * Sl - vcon * S[q])
    return out


def segment_face_centres(case, conns, ib, iconn):
    """Moment arm point of each face of a wall segment, the mean of four nodes
    (Output/OUTPUT_ClCdCm.F90:152-154, 173-175, 194-196): an array (3, nfaces), faces in the
    order of segment_wall_forces.  As the reference has it, the nodes lie at node index 1 on a
    min face and at N-1 (NI1, NJ1, NK1) -- one node layer inside the wall -- on a max face."""
    b = case.blocks[ib]
    cn = conns[b.id][iconn - 1]
    d, ci, cg, cf, is_min = _face_pairs(cn)
    X = b.xyz
    lo = [np.asarray(cf[q]) - 1 for q in range(3)]       # 0-based node of the face / of the cell's low corner
    if not is_min:
        lo[d] = lo[d] - 1                                 # Iw = NI1 on a max face
    corners = []
    for a in (0, 1):
        for e in (0, 1):
            idx = list(lo)
            o = [q for q in range(3) if q != d]
            idx[o[0]] = lo[o[0]] + a
            idx[o[1]] = lo[o[1]] + e
            corners.append(X[idx[0], idx[1], idx[2]])
    # the reference's order: (a, e) = (0, 0), (1, 0), (0, 1), (1, 1) summed left to right, / 4
    c = (((corners[0] + corners[2]) + corners[1]) + corners[3]) / 4.0
    return c.T.copy()


def wall_moments(forces, centres, ref):
    """Moment sums of Output/OUTPUT_ClCdCm.F90:250-252 over the faces of wall segments, before
    the 2/Area_Ref/B_Ref (or C_Ref) scaling and the sign of :263-265: forces and centres are
    lists of the (6, n) and (3, n) arrays of each segment; ref = (Xwc, Ywc, Zwc).  Returns
    (Cmx, Cmy, Cmz)."""
    Cmx = Cmy = Cmz = 0.0
    for F, Xc in zip(forces, centres):
        dCx, dCy, dCz = F[0] + F[3], F[1] + F[4], F[2] + F[5]
        rx, ry, rz = Xc[0] - ref[0], Xc[1] - ref[1], Xc[2] - ref[2]
        for q in range(F.shape[1]):
            Cmx = Cmx + dCy[q] * rz[q] - dCz[q] * ry[q]
            Cmz = Cmz + dCx[q] * ry[q] - dCy[q] * rx[q]
            Cmy = Cmy + dCz[q] * rx[q] - dCx[q] * rz[q]
    return Cmx, Cmy, Cmz


def moment_coefficients(Cm, area_ref, b_ref, c_ref):
    """The scaled moment coefficients of Output/OUTPUT_ClCdCm.F90:263-265."""
    Cmx, Cmy, Cmz = Cm
    return -Cmx * 2.0 / area_ref / b_ref, -Cmy * 2.0 / area_ref / b_ref, Cmz * 2.0 / area_ref / c_ref


def wall_force(case, conns, geo, fields):
    """Total (pressure + viscous) wall force."""
    Fp, Fv = wall_forces(case, conns, geo, fields)
    return Fp + Fv


def segment_cp(case, conns, fields, ib, iconn):
    """Cp = 2 (p - PPF) at the wall cells of wall segment iconn (1-based) of block ib, shaped
    over the segment's face index ranges (I, J, K)."""
    cn = conns[case.blocks[ib].id][iconn - 1]
    d, ci, cg, cf, is_min = _face_pairs(cn)
    p = _at(fields[ib]["PP"], ci)
    shape = tuple(cn.pointEnd[q] - cn.pointStart[q] + 1 for q in range(3))
    return (2.0 * (p - case.params.PPF)).reshape(shape, order="F")      # face cells run I fastest


def face_integrals(case, conns, geo, fields):
    """The quantities of trans_get_integrals (struct trans_integrals), from host arrays."""
    m_in, p0i, pi = boundary_flux(case, conns, geo, fields, 5)
    m_out, p0o, po = boundary_flux(case, conns, geo, fields, 7)
    Fp, Fv = wall_forces(case, conns, geo, fields)
    return {"mass_in": m_in, "p0_in": p0i, "p_in": pi, "mass_out": m_out, "p0_out": p0o,
            "p_out": po, "loss": (p0i - p0o) / (p0i - pi) if p0i != pi else 0.0,
            "force_p": Fp.tolist(), "force_v": Fv.tolist()}


def summary(case, conns, geo, fields):
    m_in, p0i, pi = boundary_flux(case, conns, geo, fields, 5)
    m_out, p0o, _ = boundary_flux(case, conns, geo, fields, 7)
    out = {"mass_in": m_in, "mass_out": m_out, "p0_in": p0i, "p0_out": p0o,
           "loss": (p0i - p0o) / (p0i - pi) if p0i != pi else 0.0,
           "force": wall_force(case, conns, geo, fields).tolist(),
           "cp_blade": wall_cp(case, conns, geo, fields).tolist()}
    return out


def error_table(case, conns, geo, fa, fb):
    """Relative differences of solution a from reference solution b (e.g. mixed vs FP64)."""
    sa, sb = summary(case, conns, geo, fa), summary(case, conns, geo, fb)

    def rel(x, y):
        return abs(x - y) / max(abs(y), 1e-300)
    cpa, cpb = np.array(sa["cp_blade"]), np.array(sb["cp_blade"])
    fa3, fb3 = np.array(sa["force"]), np.array(sb["force"])
    linf = 0.0
    for ib, b in enumerate(case.blocks):
        ni, nj, nk = b.dims
        sl = (slice(None), slice(G + 1, G + ni), slice(G + 1, G + nj), slice(G + 1, G + nk))
        A, B = fa[ib]["V"][sl], fb[ib]["V"][sl]
        # per equation group: density, momentum (a nearly two-dimensional flow has a tiny
        # spanwise component, so the momentum components share the scale), energy
        for grp in ((0,), (1, 2, 3), (4,)):
            scale = max(float(np.max(np.abs(B[q]))) for q in grp)
            diff = max(float(np.max(np.abs(A[q] - B[q]))) for q in grp)
            linf = max(linf, diff / scale)
    return {
        "mass_in": rel(sa["mass_in"], sb["mass_in"]),
        "mass_out": rel(sa["mass_out"], sb["mass_out"]),
        "p0_loss": rel(sa["loss"], sb["loss"]) if sb["loss"] != 0 else abs(sa["loss"]),
        "p0_loss_abs": abs(sa["loss"] - sb["loss"]),
        "blade_loading": float(np.max(np.abs(cpa - cpb)) / np.max(np.abs(cpb))),
        "force": float(np.linalg.norm(fa3 - fb3) / max(np.linalg.norm(fb3), 1e-300)),
        "field_linf": linf,
        "values_ref": {k: sb[k] for k in ("mass_in", "mass_out", "loss", "force")},
    }
