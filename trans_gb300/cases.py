"""Synthetic cases with the shapes of the benchmark configurations.

There is no public data set for this path: every grid is generated here from a seed-free
analytic description, and every initial field is the reference's KR=0 initialisation
(Input/Init.F90:94-169) plus a seeded 1e-4 relative Gaussian perturbation of the density.
"""
import math

import numpy as np

from . import abi
from .case import (Block, Case, Physical, Segment, make_params, mu_laminar_nd,
                   static_pressure_Pa)


def geometric_spacing(n_cells, first, total):
    """Node positions 0..total with geometric growth from a first spacing `first`."""
    lo, hi = 1.0 + 1e-12, 2.0
    for _ in range(200):
        r = 0.5 * (lo + hi)
        s = first * (r ** n_cells - 1.0) / (r - 1.0)
        if s > total:
            hi = r
        else:
            lo = r
    r = 0.5 * (lo + hi)
    d = first * r ** np.arange(n_cells)
    x = np.concatenate([[0.0], np.cumsum(d)])
    return x * (total / x[-1])


def _flow(XM, Tinf=288.15, p_out_ratio=None, FSTI=0.01, VisRatio=1.0):
    ps = static_pressure_Pa(Tinf)
    comm = 1.0 + 0.2 * XM * XM
    P0 = ps * comm ** 3.5
    pout = ps if p_out_ratio is None else p_out_ratio * P0
    return Physical(XM=XM, Tinf=Tinf, T0in_K=Tinf * comm, P0in_Pa=P0, Pouthub_Pa=pout,
                    FSTI=FSTI, VisRatio=VisRatio)


def channel_bump(ni=97, nj=49, nk=9, Re_L=1.0e6, XM=0.5, bump=0.08, span=0.2, **switches):
    """Channel with a sinusoidal bump on the lower wall (single block, spanwise periodic).

    x in [-L, 2L], bump y = h sin^2(pi x / L) on [0, L], top at y = L, span `span` L.
    BCs: i-min inlet (kind 5), i-max outlet (kind 7), j-min no-slip wall (kind 1),
    j-max far field (kind 2), k faces 1-to-1 onto each other (kind 9, periodic span).
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
    yw = np.where((x >= 0) & (x <= 1), bump * np.sin(math.pi * x) ** 2, 0.0)
    cf = 0.0576 * Re_L ** -0.2
    dy1 = 1.0 / (Re_L * math.sqrt(0.5 * cf))
    s = geometric_spacing(nj - 1, dy1, 1.0)
    z = np.linspace(0.0, span, nk)
    X = np.empty((ni, nj, nk, 3))
    for j in range(nj):
        X[:, j, :, 0] = x[:, None]
        X[:, j, :, 1] = (yw + (1.0 - yw) * s[j])[:, None]
    X[:, :, :, 2] = z[None, None, :]
    X /= alscale
    segs = [Segment(1, kind=5), Segment(2, kind=7), Segment(3, kind=1), Segment(4, kind=2),
            Segment(5, kind=9, blk_ex=1, blkbd_ex=6), Segment(6, kind=9, blk_ex=1, blkbd_ex=5)]
    b = Block(1, X, segs, walls=[(3, 0, 0, 0, 0)])
    return Case("channel_bump_%dx%dx%d" % (ni, nj, nk), p, [b], [X[:, 0, :, :]], ph,
                dict(Q_dst=0.05 / alscale, iterations=300))
