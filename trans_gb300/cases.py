"""Synthetic cases with the shapes of the benchmark configurations.

There is no public data set for this path: every grid is generated here from a seed-free
analytic description, and every initial field is the reference's KR=0 initialisation
(Input/Init.F90:94-169) plus a seeded 1e-4 relative Gaussian perturbation of the density.
"""
import math

import numpy as np

from . import abi
from . import detmath as dm
from .case import (Block, Case, Physical, Segment, make_params, mu_laminar_nd,
                   static_pressure_Pa)


def _ipow(r, n):
    """r**n for an integer n >= 0 by repeated squaring (platform-independent rounding)."""
    out, base = 1.0, r
    while n:
        if n & 1:
            out *= base
        base *= base
        n >>= 1
    return out


def geometric_spacing(n_cells, first, total):
    """Node positions 0..total with geometric growth from a first spacing `first`."""
    lo, hi = 1.0 + 1e-12, 2.0
    for _ in range(200):
        r = 0.5 * (lo + hi)
        s = first * (_ipow(r, n_cells) - 1.0) / (r - 1.0)
        if s > total:
            hi = r
        else:
            lo = r
    r = 0.5 * (lo + hi)
    d = first * np.array([_ipow(r, n) for n in range(n_cells)])
    x = np.concatenate([[0.0], np.cumsum(d)])
    return x * (total / x[-1])


def _flow(XM, Tinf=288.15, p_out_ratio=None, FSTI=0.01, VisRatio=1.0):
    ps = static_pressure_Pa(Tinf)
    comm = 1.0 + 0.2 * XM * XM
    P0 = ps * dm.pow(comm, 3.5)
    pout = ps if p_out_ratio is None else p_out_ratio * P0
    return Physical(XM=XM, Tinf=Tinf, T0in_K=Tinf * comm, P0in_Pa=P0, Pouthub_Pa=pout,
                    FSTI=FSTI, VisRatio=VisRatio)


def channel_bump(ni=97, nj=49, nk=9, Re_L=1.0e6, XM=0.5, bump=0.08, span=0.2, top=2, **switches):
    """Channel with a sinusoidal bump on the lower wall (single block, spanwise periodic).

    x in [-L, 2L], bump y = h sin^2(pi x / L) on [0, L], top at y = L, span `span` L.
    BCs: i-min inlet (kind 5), i-max outlet (kind 7), j-min no-slip wall (kind 1),
    j-max far field (kind 2; `top`=1 makes it a second no-slip wall, `top`=3 a symmetry plane),
    k faces 1-to-1 onto each other (kind 9, periodic span).
    """
    ph = _flow(XM)
    sw = dict(Kind_Spatial=2, Kind_Roe=1, CFL_Sub_start=5.0, CFL_Sub_end=5.0, CFL_Sub_step=1,
              Kind_Dual=2, Kchld=1, DT_LUSGS_Main=1.0e8)
    sw.update(switches)
    p0 = make_params(ph, **sw)
    # Re_L = Ref * L_grid / mu(T=1): the grid unit L_grid = 1/Alscale
    alscale = p0.Ref / (Re_L * mu_laminar_nd(p0, 1.0))
    sw["Alscale"] = alscale
    p = make_params(ph, **sw)
    x = np.linspace(-1.0, 2.0, ni)
    yw = np.where((x >= 0) & (x <= 1), bump * dm.sin(dm.pi * x) ** 2, 0.0)
    cf = 0.0576 * dm.pow(Re_L, -0.2)
    dy1 = 1.0 / (Re_L * math.sqrt(0.5 * cf))
    s = geometric_spacing(nj - 1, dy1, 1.0)
    z = np.linspace(0.0, span, nk)
    X = np.empty((ni, nj, nk, 3))
    for j in range(nj):
        X[:, j, :, 0] = x[:, None]
        X[:, j, :, 1] = (yw + (1.0 - yw) * s[j])[:, None]
    X[:, :, :, 2] = z[None, None, :]
    X /= alscale
    if top not in (1, 2, 3):
        raise ValueError("top boundary: kind 2 (far field), 1 (wall) or 3 (symmetry)")
    segs = [Segment(1, kind=5), Segment(2, kind=7), Segment(3, kind=1), Segment(4, kind=top),
            Segment(5, kind=9, blk_ex=1, blkbd_ex=6), Segment(6, kind=9, blk_ex=1, blkbd_ex=5)]
    b = Block(1, X, segs, walls=[(3, 0, 0, 0, 0)] + ([(4, 0, 0, 0, 0)] if top == 1 else []))
    walls = [X[:, 0, :, :]] + ([X[:, -1, :, :]] if top == 1 else [])
    return Case("channel_bump_%dx%dx%d" % (ni, nj, nk) + {1: "_walls", 2: "", 3: "_symm"}[top], p, [b], walls, ph,
                dict(Q_dst=0.05 / alscale, iterations=300))


def annular_sector(ni=25, nj=13, nk=9, sector_deg=10.0, r_hub=1.0, r_tip=1.5, Re_L=1.0e6, XM=0.4,
                   p_ratio=0.95, rpm=0.0, casing_kindsub=0, **switches):
    """Annular duct sector with rotational periodicity (single block): x in [-1, 2] axial (i),
    r in [r_hub, r_tip] (j), theta in [0, sector] (k) about the x axis.  BCs: i-min inlet
    (kind 5), i-max outlet (kind 7, radial-equilibrium recurrence over r), hub and casing
    no-slip walls (kind 1), k faces 1-to-1 onto each other (kind 9) across the sector, so the
    interface rotates (v, w) and the gradients by rotateAngle = +-sector
    (Input/PLOT3DReadInit.F90:157-160 with nblade = 360/sector, one passage).

    rpm: the frame's rotation about the x axis (omega(1) of the dimension file, in rev/min);
    the hub turns with the frame, and the casing does too unless casing_kindsub = 1, which
    makes it a wall at rest in the absolute frame (BC_Wall.F90:46-52)."""
    nblade = int(round(360.0 / sector_deg))
    ph = _flow(XM, p_out_ratio=p_ratio)
    ph.nblade, ph.npassage = nblade, 1
    ph.omega_rpm = (float(rpm), 0.0, 0.0)
    sw = dict(Kind_Spatial=3, Kind_Roe=3, CFL_Sub_start=2.0, CFL_Sub_end=2.0, CFL_Sub_step=1,
              Kind_Dual=2, Kchld=1, DT_LUSGS_Main=1.0e8)
    sw.update(switches)
    p0 = make_params(ph, **sw)
    alscale = p0.Ref / (Re_L * mu_laminar_nd(p0, 1.0))
    sw["Alscale"] = alscale
    p = make_params(ph, **sw)
    x = np.linspace(-1.0, 2.0, ni)
    r = r_hub + (r_tip - r_hub) * (0.5 - 0.5 * dm.cos(dm.pi * np.linspace(0.0, 1.0, nj)))
    th = np.linspace(0.0, 2.0 * dm.pi / nblade, nk)
    X = np.empty((ni, nj, nk, 3))
    X[..., 0] = x[:, None, None]
    X[..., 1] = r[None, :, None] * dm.cos(th)[None, None, :]
    X[..., 2] = r[None, :, None] * dm.sin(th)[None, None, :]
    X /= alscale
    # k-min ghosts take the k-max cells (one sector further round): their (v, w) rotate back by
    # the sector angle, V(3) = cos a vy + sin a vz with a = +sector (BC/BC_P2P.F90:69-94)
    segs = [Segment(1, kind=5), Segment(2, kind=7), Segment(3, kind=1), Segment(4, kind=1, kindsub=casing_kindsub),
            Segment(5, kind=9, blk_ex=1, blkbd_ex=6, period=1), Segment(6, kind=9, blk_ex=1, blkbd_ex=5, period=-1)]
    b = Block(1, X, segs, walls=[(3, 0, 0, 0, 0), (4, 0, 0, 0, 0)])
    walls = [X[:, 0, :, :], X[:, -1, :, :]]
    return Case("annular_sector_%dx%dx%d" % (ni, nj, nk), p, [b], walls, ph,
                dict(Q_dst=0.05 / alscale, iterations=300))


# --------------------------------------------------------------------------------------------
# Linear compressor cascade, five blocks (O-grid around the blade + inlet/outlet H blocks +
# two passage blocks), pitch-periodic 1-to-1 interfaces, endwalls.
# --------------------------------------------------------------------------------------------
def _blade(camber_deg=40.0, stagger_deg=30.0, thick=0.08, rot_deg=0.0):
    """Circular-arc camber line (chord 1), elliptic-nosed thickness 2*t*sqrt(x(1-x)),
    staggered, then rotated by rot_deg.  Returns functions of the chord fraction."""
    th = dm.radians(camber_deg)
    R = 1.0 / (2.0 * dm.sin(th / 2))
    yc0 = -R * dm.cos(th / 2)
    ca, sa = dm.cos(dm.radians(stagger_deg + rot_deg)), dm.sin(dm.radians(stagger_deg + rot_deg))

    def camber(xi):
        z = np.sqrt(R * R - (xi - 0.5) ** 2) + yc0
        dz = -(xi - 0.5) / np.sqrt(R * R - (xi - 0.5) ** 2)
        return z, dz

    def surface(xi, side):
        z, dz = camber(xi)
        nrm = np.sqrt(1.0 + dz * dz)
        nx, nz = -dz / nrm, 1.0 / nrm              # unit normal towards +z (suction side)
        h = thick * np.sqrt(np.clip(xi * (1.0 - xi), 0.0, None))
        px = xi + side * h * nx
        pz = z + side * h * nz
        return ca * px - sa * pz, sa * px + ca * pz

    def mean(xi):
        z, dz = camber(xi)
        return ca * xi - sa * z, sa * xi + ca * z

    return surface, mean


def _stretch(n, first_frac):
    """n cells from 0 to 1 with geometric growth from first_frac."""
    return geometric_spacing(n, first_frac, 1.0)


def _two_sided(n, first):
    """n cells on [0,1] clustered at both ends with first spacing `first` (n even)."""
    h = geometric_spacing(n // 2, first, 0.5)
    return np.concatenate([h, 1.0 - h[::-1][1:]])


# The five-block cascade at the sizes of the benchmark configuration: O-block 257x49x65 and
# passage blocks 97x33x65 as stated.  With 1-to-1 interfaces the H-blocks' pitchwise node count
# is forced: their face towards the blade is the two passage blocks' pitch edges plus the
# O-block's leading-edge (or trailing-edge) cap, 2*npitch + nle = 2*32 + 32 = 96 cells, and the
# O-block loop is 2*ns + 2*nte + nle = 2*96 + 2*16 + 32 = 256 cells.  (H-blocks of 41 pitchwise
# nodes would force passage blocks of at most 121x17 nodes, 10% fewer cells in all.)  Interior
# cells: 786,432 + 2 x 393,216 + 2 x 196,608 = 1,966,080.
CASCADE_CONFIG2 = dict(ns=96, npitch=32, nle=32, nte=16, nr=48, nh=64, nk=64)


def cascade(nle=8, nte=4, ns=120, npitch=16, nr=48, nh=64, nk=64, Re_c=1.0e6, XM=0.6, inflow_deg=40.0,
            p_ratio=0.85, pitch=0.8, span=1.0, radius=10.0, cluster=1.0, **switches):
    """Linear compressor cascade passage with the block structure of a turbomachinery mesh:
    O-block (2*nte+2*ns+nle around x nr x nk) on a circular-arc blade (8% thick, 40 deg camber,
    30 deg stagger), inlet/outlet H-blocks (nh x (2*npitch+nle) x nk) and two passage blocks
    (ns x npitch x nk).  The geometry is rotated so that the inflow (inflow_deg from axial) is
    along +x, since the total-pressure inlet (BC/BC_Inlet.F90:54-56) imposes axial velocity;
    the passage sits at mean radius `radius` chords, which the outlet radial-equilibrium
    recurrence (BC/BC_Outlet.F90:57-70) reads.  Outlet static pressure = p_ratio x inlet total.
    """
    ph = _flow(XM, p_out_ratio=p_ratio)
    sw = dict(Kind_Spatial=3, Kind_Roe=3, CFL_Sub_start=10.0, CFL_Sub_end=10.0, CFL_Sub_step=1,
              Kind_Dual=2, Kchld=1, DT_LUSGS_Main=1.0e8, gama_max=0.0463783, gama_min=0.0)
    sw.update(switches)
    p0 = make_params(ph, **sw)
    alscale = p0.Ref / (Re_c * mu_laminar_nd(p0, 1.0))
    sw["Alscale"] = alscale
    p = make_params(ph, **sw)
    surf, mean = _blade(rot_deg=-inflow_deg)
    # chord-fraction parameters of the blade loop segments
    xi_l, xi_t = 0.02, 0.98
    t = np.linspace(0.0, 1.0, ns + 1)
    u = 0.5 * (1.0 - dm.cos(dm.pi * t))
    if cluster != 1.0:          # blend the cosine clustering with uniform spacing
        u = cluster * u + (1.0 - cluster) * t
    xi_side = xi_l + (xi_t - xi_l) * u                   # LE -> TE
    # mean line of the passage: camber line on the blade, continued with the end slopes
    xm_le, ym_le = mean(np.array(0.0))
    xm_te, ym_te = mean(np.array(1.0))
    xq = np.linspace(0.0, 1.0, 401)
    mx, my = mean(xq)
    s_le = (my[1] - my[0]) / (mx[1] - mx[0])
    s_te = (my[-1] - my[-2]) / (mx[-1] - mx[-2])
    L_up, L_dn = 1.0, 1.0
    h = 0.15
    dlt = 0.08
    xa, xb = float(mx[0]) - dlt, float(mx[-1]) + dlt

    def ymean(x):
        x = np.asarray(x, float)
        y = np.interp(x, mx, my)
        up = x < mx[0]
        # upstream: slope decays from the leading-edge slope to 0 at the inlet
        d = x - mx[0]
        y = np.where(up, my[0] + s_le * d * (1.0 + d / (2.0 * (L_up + dlt))), y)
        dn = x > mx[-1]
        y = np.where(dn, my[-1] + s_te * (x - mx[-1]), y)
        return y

    # ---- O-block loop (outer rectangle in (x, eta)) and blade loop, i = 1..NIo ----
    xs_p, ys_p = surf(xi_side[::-1], -1.0)               # pressure side TE -> LE
    xs_s, ys_s = surf(xi_side, +1.0)                     # suction side LE -> TE
    # TE caps (pressure side from xi=1 to xi_t, suction from xi_t to 1) and LE cap
    cap_t = np.linspace(1.0, xi_t, nte + 1)
    xtp, ytp = surf(cap_t, -1.0)
    xts, yts = surf(cap_t[::-1], +1.0)
    ang = np.linspace(0.0, 1.0, nle + 1)
    xi_cap = np.where(ang <= 0.5, xi_l * (1 - 2 * ang), xi_l * (2 * ang - 1))
    side = np.where(ang < 0.5, -1.0, 1.0)
    xlc, ylc = surf(xi_cap, side)
    bx = np.concatenate([xtp, xs_p[1:], xlc[1:], xs_s[1:], xts[1:]])
    by = np.concatenate([ytp, ys_p[1:], ylc[1:], ys_s[1:], yts[1:]])
    # outer loop: x positions of the sides follow the blade points, rescaled to [xa, xb]
    xr = (xs_s - xs_s[0]) / (xs_s[-1] - xs_s[0])
    x_top = xa + (xb - xa) * xr
    eta_te = np.linspace(0.0, -h, nte + 1)
    eta_le = np.linspace(-h, h, nle + 1)
    ox = np.concatenate([np.full(nte + 1, xb), x_top[::-1][1:], np.full(nle, xa), x_top[1:], np.full(nte, xb)])
    oe = np.concatenate([eta_te, np.full(ns, -h), eta_le[1:], np.full(ns, h), (-eta_te[::-1])[1:]])
    oy = ymean(ox) + oe
    nio = len(bx)
    assert nio == 2 * nte + 2 * ns + nle + 1 and len(ox) == nio
    bx[-1], by[-1] = bx[0], by[0]
    first = 1.0 / (Re_c * math.sqrt(0.5 * 0.0576 * dm.pow(Re_c, -0.2)))
    dist = dm.hypot(ox - bx, oy - by)
    sig = _stretch(nr, first / float(np.min(dist)))
    z = _two_sided(nk, first / span) * span
    Xo = np.empty((nio, nr + 1, nk + 1, 3))
    Xo[:, :, :, 0] = (bx[:, None] + (ox - bx)[:, None] * sig[None, :])[:, :, None]
    Xo[:, :, :, 1] = (by[:, None] + (oy - by)[:, None] * sig[None, :])[:, :, None]
    Xo[:, :, :, 2] = z[None, None, :]
    # ---- passage and H blocks on the (x, eta) lattice ----
    eta_p = h + (pitch / 2 - h) * _stretch(npitch, 0.03)          # eta of P1 from h to pitch/2
    eta_h = np.concatenate([-eta_p[::-1], eta_le[1:-1], eta_p])   # full pitch, 2*npitch+nle cells

    def lattice(xv, etav):
        X = np.empty((len(xv), len(etav), nk + 1, 3))
        X[:, :, :, 0] = xv[:, None, None]
        X[:, :, :, 1] = (ymean(xv)[:, None] + etav[None, :])[:, :, None]
        X[:, :, :, 2] = z[None, None, :]
        return X

    dx_a = float(x_top[1] - x_top[0])
    x_in = xa - L_up
    x_up = xa - L_up * _stretch(nh, dx_a / L_up)[::-1]
    x_up[0] = x_in
    x_dn = xb + L_dn * _stretch(nh, float(x_top[-1] - x_top[-2]) / L_dn)
    Xh1 = lattice(x_up, eta_h)
    Xh2 = lattice(x_dn, eta_h)
    Xp1 = lattice(x_top, eta_p)
    Xp2 = lattice(x_top, -eta_p[::-1])
    scale = 1.0 / alscale
    blocks_xyz = []
    for X in (Xo, Xh1, Xh2, Xp1, Xp2):
        Y = X.copy()
        Y[..., 1] += radius
        blocks_xyz.append(Y * scale)
    Xo, Xh1, Xh2, Xp1, Xp2 = blocks_xyz
    nlo = 2 * npitch + nle
    S = Segment
    # O = 1, H1 = 2, H2 = 3, P1 = 4, P2 = 5
    o_segs = [S(1, kind=9, blk_ex=1, blkbd_ex=2), S(2, kind=9, blk_ex=1, blkbd_ex=1), S(3, kind=1),
              S(4, 1, nte, kind=9, blk_ex=3, blkbd_ex=3, lrev_a=1),
              S(4, nte + 1, nte + ns, kind=9, blk_ex=5, blkbd_ex=4, lrev_a=1),
              S(4, nte + ns + 1, nte + ns + nle, kind=9, blk_ex=2, blkbd_ex=3),
              S(4, nte + ns + nle + 1, nte + 2 * ns + nle, kind=9, blk_ex=4, blkbd_ex=3),
              S(4, nte + 2 * ns + nle + 1, 2 * nte + 2 * ns + nle, kind=9, blk_ex=3, blkbd_ex=4, lrev_a=1),
              S(5, kind=1), S(6, kind=1)]
    h1_segs = [S(1, kind=5),
               S(2, 1, npitch, kind=9, blk_ex=5, blkbd_ex=1),
               S(2, npitch + 1, npitch + nle, kind=9, blk_ex=1, blkbd_ex=6),
               S(2, npitch + nle + 1, nlo, kind=9, blk_ex=4, blkbd_ex=1),
               S(3, kind=9, blk_ex=2, blkbd_ex=6), S(4, kind=9, blk_ex=2, blkbd_ex=5),
               S(5, kind=1), S(6, kind=1)]
    h2_segs = [S(2, kind=7),
               S(1, 1, npitch, kind=9, blk_ex=5, blkbd_ex=2),
               S(1, npitch + 1, npitch + nte, kind=9, blk_ex=1, blkbd_ex=4, lrev_a=1),
               S(1, npitch + nte + 1, npitch + nle, kind=9, blk_ex=1, blkbd_ex=8, lrev_a=1),
               S(1, npitch + nle + 1, nlo, kind=9, blk_ex=4, blkbd_ex=2),
               S(3, kind=9, blk_ex=3, blkbd_ex=7), S(4, kind=9, blk_ex=3, blkbd_ex=6),
               S(5, kind=1), S(6, kind=1)]
    p1_segs = [S(1, kind=9, blk_ex=2, blkbd_ex=4), S(2, kind=9, blk_ex=3, blkbd_ex=5),
               S(3, kind=9, blk_ex=1, blkbd_ex=7), S(4, kind=9, blk_ex=5, blkbd_ex=3),
               S(5, kind=1), S(6, kind=1)]
    p2_segs = [S(1, kind=9, blk_ex=2, blkbd_ex=2), S(2, kind=9, blk_ex=3, blkbd_ex=2),
               S(3, kind=9, blk_ex=4, blkbd_ex=4), S(4, kind=9, blk_ex=1, blkbd_ex=5, lrev_a=1),
               S(5, kind=1), S(6, kind=1)]
    end = [(5, 0, 0, 0, 0), (6, 0, 0, 0, 0)]
    blocks = [Block(1, Xo, o_segs, walls=[(3, 0, 0, 0, 0)] + end), Block(2, Xh1, h1_segs, walls=end),
              Block(3, Xh2, h2_segs, walls=end), Block(4, Xp1, p1_segs, walls=end),
              Block(5, Xp2, p2_segs, walls=end)]
    surfaces = [Xo[:, 0, :, :]] + [X[:, :, kk, :] for X in blocks_xyz for kk in (0, -1)]
    name = "cascade_5blk_%dcells" % sum(int(np.prod([d - 1 for d in b.dims])) for b in blocks)
    return Case(name, p, blocks, surfaces, ph, dict(Q_dst=0.02 / alscale, chord=scale, pitch=pitch * scale,
                                                    p_ratio=p_ratio))


# --------------------------------------------------------------------------------------------
# Square cylinder, one O-block, time-accurate DES (dual time stepping).
# --------------------------------------------------------------------------------------------
def _square_loop(n_side, half):
    """Nodes around a square of half-width `half` (closed loop, counterclockwise from the
    middle of the rear face), `n_side` cells per side: 4*n_side + 1 nodes, last = first."""
    corners = [(half, half), (-half, half), (-half, -half), (half, -half)]
    pts = []
    # rear face upper half: (half, 0) -> (half, half)
    h = n_side // 2
    t = np.linspace(0.0, 1.0, h + 1)
    pts.append(np.stack([np.full(h + 1, half), t * half], axis=1))
    prev = corners[0]
    for cnr in corners[1:]:
        t = np.linspace(0.0, 1.0, n_side + 1)[1:]
        pts.append(np.stack([prev[0] + (cnr[0] - prev[0]) * t, prev[1] + (cnr[1] - prev[1]) * t], axis=1))
        prev = cnr
    t = np.linspace(0.0, 1.0, n_side - h + 1)[1:]
    pts.append(np.stack([np.full(n_side - h, half), -half + t * half], axis=1))
    return np.concatenate(pts, axis=0)


def _rect_loop(n_side, x0, x1, y0, y1, xc=0.0):
    """The same node count around the rectangle [x0,x1]x[y0,y1], side by side with
    _square_loop (rear face <-> outflow side, etc.)."""
    h = n_side // 2
    pts = []
    t = np.linspace(0.0, 1.0, h + 1)
    pts.append(np.stack([np.full(h + 1, x1), t * y1], axis=1))
    corners = [(x1, y1), (x0, y1), (x0, y0), (x1, y0)]
    prev = corners[0]
    for cnr in corners[1:]:
        t = np.linspace(0.0, 1.0, n_side + 1)[1:]
        pts.append(np.stack([prev[0] + (cnr[0] - prev[0]) * t, prev[1] + (cnr[1] - prev[1]) * t], axis=1))
        prev = cnr
    t = np.linspace(0.0, 1.0, n_side - h + 1)[1:]
    pts.append(np.stack([np.full(n_side - h, x1), y0 + t * (0.0 - y0)], axis=1))
    return np.concatenate(pts, axis=0)


def square_cylinder(ni=385, nj=257, nk=129, Re_D=2.0e4, XM=0.2, span=4.0, box=(-10.0, 20.0, -10.0, 10.0),
                    dt_UD=0.005, perturbation=0.01, **switches):
    """Wake of a square cylinder (side D = 1): one O-block around it, i around the section
    (wrapping through a self 1-to-1 cut: i-min onto i-max), j from the wall (kind 1) to a
    rectangular outer boundary `box` (far field, kind 2), k spanwise over `span` D (periodic
    1-to-1).  DES (Kind_Hybrid = 3, Kind_SubHY = 0) with dual time stepping: Kchld
    sub-iterations per physical step dt*U/D = dt_UD.  The initial field is the freestream with
    a seeded `perturbation` relative Gaussian perturbation of the velocity."""
    if (ni - 1) % 4:
        raise ValueError("ni - 1 must be a multiple of 4 (cells per side of the square)")
    ph = _flow(XM)
    sw = dict(Kind_Spatial=3, Kind_Roe=3, Kind_Hybrid=3, Kind_SubHY=0, CFL_Sub_start=5.0, CFL_Sub_end=5.0,
              CFL_Sub_step=1, Kind_Dual=2, Kchld=10, DT_LUSGS_Main=1.0, gama_max=0.0463783, gama_min=0.0)
    sw.update(switches)
    p0 = make_params(ph, **sw)
    alscale = p0.Ref / (Re_D * mu_laminar_nd(p0, 1.0))
    sw["Alscale"] = alscale
    # the physical time step in the reference's units (length 1/alscale = D, velocity Vref)
    if "DT_LUSGS_Main" not in switches:
        sw["DT_LUSGS_Main"] = dt_UD / alscale
    p = make_params(ph, **sw)
    n_side = (ni - 1) // 4
    inner = _square_loop(n_side, 0.5)
    outer = _rect_loop(n_side, *box)
    # wall-normal distribution: geometric from y+ ~ 1 at the wall, the same parameter on
    # every i-line (transfinite interpolation between the square and the rectangle)
    cf = 0.0576 * dm.pow(Re_D, -0.2)
    dy1 = 1.0 / (Re_D * math.sqrt(0.5 * cf))
    reach = float(np.mean(np.hypot(outer[:, 0] - inner[:, 0], outer[:, 1] - inner[:, 1])))
    eta = geometric_spacing(nj - 1, dy1 / reach, 1.0)
    z = np.linspace(0.0, span, nk)
    X = np.empty((ni, nj, nk, 3))
    for j in range(nj):
        X[:, j, :, 0] = (inner[:, 0] + eta[j] * (outer[:, 0] - inner[:, 0]))[:, None]
        X[:, j, :, 1] = (inner[:, 1] + eta[j] * (outer[:, 1] - inner[:, 1]))[:, None]
    X[:, :, :, 2] = z[None, None, :]
    X /= alscale
    segs = [Segment(1, kind=9, blk_ex=1, blkbd_ex=2), Segment(2, kind=9, blk_ex=1, blkbd_ex=1),
            Segment(3, kind=1), Segment(4, kind=2),
            Segment(5, kind=9, blk_ex=1, blkbd_ex=6), Segment(6, kind=9, blk_ex=1, blkbd_ex=5)]
    b = Block(1, X, segs, walls=[(3, 0, 0, 0, 0)])
    return Case("square_cylinder_%dx%dx%d" % (ni, nj, nk), p, [b], [X[:, 0, :, :]], ph,
                dict(Q_dst=0.05 / alscale, velocity_noise=perturbation, D=1.0 / alscale, dt_UD=dt_UD,
                     steps=2000))
