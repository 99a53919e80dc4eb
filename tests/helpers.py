"""Shared helpers of the test-suite: cases, masks over the ghost-padded arrays, comparisons."""
import hashlib

import numpy as np

from trans_gb300 import case as C
from trans_gb300 import cases

G = 2


def small_channel(ni=25, nj=17, nk=6, **sw):
    c = cases.channel_bump(ni=ni, nj=nj, nk=nk, **sw)
    conns, geo = C.compute_geometry(c)
    st = C.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    return c, conns, geo, st


# rotating annular sector: 2000 rev/min gives a blade speed omega*r of about 0.27 of the axial
# velocity at the casing; the casing is at rest in the absolute frame (Kindsub_BC = 1)
SMALL_ANNULAR = dict(ni=17, nj=11, nk=6, rpm=2000.0, casing_kindsub=1)


def small_annular(**sw):
    c = cases.annular_sector(**SMALL_ANNULAR, **sw)
    conns, geo = C.compute_geometry(c)
    st = C.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    return c, conns, geo, st


def small_case(kind, **sw):
    """The small case of a golden fixture's kind: channel, cascade or annular."""
    return {"channel": small_channel, "cascade": small_cascade, "annular": small_annular}[kind](**sw)


def interior(dims):
    ni, nj, nk = dims
    m = np.zeros((ni + 5, nj + 5, nk + 5), bool, order="F")
    m[G + 1:G + ni, G + 1:G + nj, G + 1:G + nk] = True
    return m


def face_ghosts(dims, layers=3):
    """Ghost cells that lie across exactly one face (not edges or corners)."""
    ni, nj, nk = dims
    m = np.zeros((ni + 5, nj + 5, nk + 5), bool, order="F")
    I, J, K = slice(G + 1, G + ni), slice(G + 1, G + nj), slice(G + 1, G + nk)
    for L in range(1, layers + 1):
        m[G + 1 - L, J, K] = True; m[G + ni - 1 + L, J, K] = True
        m[I, G + 1 - L, K] = True; m[I, G + nj - 1 + L, K] = True
        m[I, J, G + 1 - L] = True; m[I, J, G + nk - 1 + L] = True
    return m


def rel_err(a, b, mask):
    """max |a-b| / max |b| over the masked cells, per leading component."""
    a = np.asarray(a); b = np.asarray(b)
    lead = a.shape[:-3]
    a2 = a.reshape((-1,) + a.shape[-3:])
    b2 = b.reshape((-1,) + b.shape[-3:])
    out = []
    for q in range(a2.shape[0]):
        x, y = a2[q][mask], b2[q][mask]
        scale = np.max(np.abs(y)) if y.size else 0.0
        d = np.max(np.abs(x - y)) if y.size else 0.0
        out.append(d / scale if scale > 0 else d)
    return np.array(out).reshape(lead) if lead else out[0]


def bit_equal_fraction(a, b, mask):
    a2 = np.asarray(a).reshape((-1,) + np.asarray(a).shape[-3:])
    b2 = np.asarray(b).reshape((-1,) + np.asarray(b).shape[-3:])
    eq = tot = 0
    for q in range(a2.shape[0]):
        x, y = a2[q][mask], b2[q][mask]
        eq += int(np.sum(x.view(np.int64) == y.view(np.int64)))
        tot += x.size
    return eq / max(tot, 1)


SMALL_CASCADE = dict(nle=4, nte=2, ns=8, npitch=3, nr=6, nh=6, nk=4)


def small_cascade(**sw):
    c = cases.cascade(**SMALL_CASCADE, **sw)
    conns, geo = C.compute_geometry(c)
    st = C.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    return c, conns, geo, st


def inputs_digest(c, geo, st):
    """SHA-256 over every geometry and state array handed to the solver, in a fixed order:
    equal digests mean bit-identical inputs (the host set-up is platform-independent)."""
    h = hashlib.sha256()
    for b in c.blocks:
        for name in sorted(geo[b.id]):
            h.update(np.ascontiguousarray(geo[b.id][name]).tobytes())
        for name in sorted(st[b.id]):
            h.update(np.ascontiguousarray(st[b.id][name]).tobytes())
    return h.hexdigest()
