"""Integrated quantities on the host (trans_gb300.integrals): known answers on uniform states and
a face-by-face scalar restatement of the reference's output routines on a perturbed state.

The library computes the same sums on the device (trans_get_integrals); the GPU tests hold the
device sums against these host sums.  Tolerances: known answers to 1e-13 relative (a sum of a
few hundred terms), the scalar restatement to 1e-13 relative (same expressions, another
summation order).
"""
import math

import numpy as np

from helpers import G, small_cascade, small_channel
from trans_gb300 import integrals
from trans_gb300.case import face_cells


def _fields(st, c):
    return [{k: st[b.id][k] for k in ("V", "PP", "T")} for b in c.blocks]


def _uniform(c, st, u=(0.5, 0.0, 0.0), rho=1.0, p=None):
    p = c.params.PPF if p is None else p
    for b in c.blocks:
        s = st[b.id]
        V = s["V"]
        V[...] = 0.0
        V[0][...] = rho
        for q in range(3):
            V[q + 1][...] = rho * u[q]
        V[4][...] = p / 0.4 + 0.5 * rho * sum(x * x for x in u)
        s["PP"][...] = p
        s["T"][...] = 1.0


def test_uniform_state_known_answers():
    """Uniform state with p = PPF: p0 = p (1 + 0.2 M^2)^3.5 on both sides, no loss, no pressure
    force, Cp = 0, mass flow = rho u . sum(S) of the inlet faces."""
    c, conns, geo, st = small_channel()
    u = (0.5, 0.0, 0.0)
    _uniform(c, st, u)
    r = integrals.face_integrals(c, conns, geo, _fields(st, c))
    P = c.params
    M2 = (u[0] ** 2) / (1.4 * P.PPF / 1.0)
    p0 = P.PPF * (1.0 + 0.2 * M2) ** 3.5
    assert abs(r["p0_in"] - p0) <= 1e-13 * p0
    assert abs(r["p0_out"] - p0) <= 1e-13 * p0
    assert abs(r["p_in"] - P.PPF) <= 1e-13 * P.PPF
    assert abs(r["loss"]) <= 1e-10
    assert max(abs(x) for x in r["force_p"]) == 0.0
    sx = 0.0
    for cn in conns[c.blocks[0].id]:
        if cn.BCType == 5:
            I, J, K = face_cells(cn)
            sx += float(np.sum(geo[c.blocks[0].id]["SD"][0, 0][I + G, J + G, K + G]))
    assert abs(r["mass_in"] - 0.5 * sx) <= 1e-13 * abs(0.5 * sx)
    cp = integrals.segment_cp(c, conns, _fields(st, c), 0, 3)
    assert cp.shape == (24, 1, 5) and np.all(cp == 0.0)


def test_uniform_state_at_rest_has_no_viscous_force():
    c, conns, geo, st = small_cascade()
    _uniform(c, st, (0.0, 0.0, 0.0), p=1.1 * c.params.PPF)
    Fp, Fv = integrals.wall_forces(c, conns, geo, _fields(st, c))
    assert np.all(Fv == 0.0)
    # a uniform excess pressure on the walls of every block: (p - PPF) times the walls' sum(S Sgn)
    assert np.all(np.isfinite(Fp))


def _scalar_integrals(c, conns, geo, fields):
    """Face-by-face loops over every inlet, outlet and wall face (the reference's loops)."""
    P = c.params
    acc = np.zeros(12)
    for ib, b in enumerate(c.blocks):
        g = geo[b.id]
        V, PP, T = fields[ib]["V"], fields[ib]["PP"], fields[ib]["T"]
        for cn in conns[b.id]:
            if cn.BCType not in (1, 5, 7):
                continue
            d = cn.IJKDirect - 1
            is_min = cn.pointStart[d] == 1
            for K in range(cn.pointStart[2], cn.pointEnd[2] + 1):
                for J in range(cn.pointStart[1], cn.pointEnd[1] + 1):
                    for I in range(cn.pointStart[0], cn.pointEnd[0] + 1):
                        f = [I, J, K]
                        inner, ghost = list(f), list(f)
                        if is_min:
                            ghost[d] -= 1
                        else:
                            inner[d] -= 1
                        ci = tuple(x + G for x in inner)
                        cg = tuple(x + G for x in ghost)
                        cf = tuple(x + G for x in f)
                        S = [g["SD"][d, q][cf] for q in range(3)]
                        if cn.BCType in (5, 7):
                            w1, w2 = g["VOL"][cg], g["VOL"][ci]
                            ws = w1 + w2
                            rho = (w1 * V[0][ci] + w2 * V[0][cg]) / ws
                            ru = [(w1 * V[q][ci] + w2 * V[q][cg]) / ws for q in (1, 2, 3)]
                            p = (w1 * PP[ci] + w2 * PP[cg]) / ws
                            flux = ru[0] * S[0] + ru[1] * S[1] + ru[2] * S[2]
                            mf = flux if (cn.BCType == 5) == is_min else -flux
                            M2 = ((ru[0] ** 2 + ru[1] ** 2 + ru[2] ** 2) / (rho * rho)) / (1.4 * p / rho)
                            p0 = p * (1.0 + 0.2 * M2) ** 3.5
                            o = 0 if cn.BCType == 5 else 3
                            acc[o] += mf; acc[o + 1] += mf * p0; acc[o + 2] += mf * p
                        else:
                            Sl = g["GRAD"][d][cf]
                            n = [x / Sl for x in S]
                            sgn = -1.0 if is_min else 1.0
                            for q in range(3):
                                acc[6 + q] += (PP[ci] - P.PPF) * n[q] * Sl * sgn
                            TT = T[ci]
                            mu = (1.0 + P.Csthlnd) / (TT * P.Csth1 + P.Csthlnd) * (P.Csth1 * TT) ** 1.5
                            uu = [V[q + 1][ci] / V[0][ci] for q in range(3)]
                            vcon = sum(uu[q] * n[q] * Sl for q in range(3))
                            tau = mu / g["DST"][ci] / P.Ref
                            for q in range(3):
                                acc[9 + q] += tau * (uu[q] * Sl - vcon * n[q])
    return acc


def test_face_integrals_match_scalar_loops():
    c, conns, geo, st = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    rng = np.random.default_rng(3)
    for b in c.blocks:
        s = st[b.id]
        s["V"][...] *= 1.0 + 0.01 * rng.standard_normal(s["V"].shape)
        s["PP"][...] *= 1.0 + 0.01 * rng.standard_normal(s["PP"].shape)
        s["T"][...] *= 1.0 + 0.01 * rng.standard_normal(s["T"].shape)
    f = _fields(st, c)
    r = integrals.face_integrals(c, conns, geo, f)
    a = _scalar_integrals(c, conns, geo, f)
    assert math.isclose(r["mass_in"], a[0], rel_tol=1e-13)
    assert math.isclose(r["p0_in"], a[1] / a[0], rel_tol=1e-13)
    assert math.isclose(r["p_in"], a[2] / a[0], rel_tol=1e-13)
    assert math.isclose(r["mass_out"], a[3], rel_tol=1e-13)
    assert math.isclose(r["p0_out"], a[4] / a[3], rel_tol=1e-13)
    scale_p = max(abs(x) for x in a[6:9])
    scale_v = max(abs(x) for x in a[9:12])
    assert scale_p > 0 and scale_v > 0
    assert max(abs(x - y) for x, y in zip(r["force_p"], a[6:9])) <= 1e-13 * scale_p
    assert max(abs(x - y) for x, y in zip(r["force_v"], a[9:12])) <= 1e-13 * scale_v


def test_wall_moments_are_minus_r_cross_f():
    """The moment sums of Output/OUTPUT_ClCdCm.F90:250-252 are minus the sum of r x F, with r
    from the reference point to the face centre; the face centre is the mean of four nodes at
    node index 1 on a min face and N-1 on a max face (the reference's Iw = NI1)."""
    from trans_gb300 import case as CS
    c, conns, geo, st = small_channel()
    b = c.blocks[0]
    X = b.xyz
    ni, nj, nk = b.dims
    rng = np.random.default_rng(3)
    for ic, cn in enumerate(conns[b.id], start=1):
        if cn.BCType != 1:
            continue
        Xc = integrals.segment_face_centres(c, conns, 0, ic)
        I, J, K = face_cells(cn)
        d = cn.IJKDirect - 1
        node = 0 if cn.pointStart[d] == 1 else [ni, nj, nk][d] - 2
        q = 0
        idx = [I - 1, J - 1, K - 1]
        idx[d] = np.full_like(idx[d], node)
        o = [a for a in range(3) if a != d]
        ref = np.zeros((3, len(I)))
        for a in (0, 1):
            for e in (0, 1):
                jdx = list(idx)
                jdx[o[0]] = idx[o[0]] + a
                jdx[o[1]] = idx[o[1]] + e
                ref += X[jdx[0], jdx[1], jdx[2]].T
        np.testing.assert_allclose(Xc, ref / 4.0, rtol=0, atol=1e-14 * np.max(np.abs(X)))
        F = rng.standard_normal((6, Xc.shape[1]))
        r0 = (0.3, -0.2, 0.1)
        Cm = integrals.wall_moments([F], [Xc], r0)
        r = Xc - np.array(r0)[:, None]
        cross = np.cross(r.T, (F[:3] + F[3:]).T).sum(axis=0)
        np.testing.assert_allclose(Cm, -cross, rtol=1e-12, atol=1e-12)
        q += 1
