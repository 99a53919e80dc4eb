"""Case generator and caller-side set-up: block connectivity, interface node matching, metrics."""
import numpy as np
import pytest

from trans_gb300 import case as C
from trans_gb300 import cases

SMALL_CASCADE = dict(nle=4, nte=2, ns=8, npitch=3, nr=6, nh=6, nk=4)


def _face_centre(X, c, i, j, k):
    """Centre of the boundary face of cell (i,j,k) on connection c (node arrays are 0-based)."""
    d = c.IJKDirect - 1
    n = [i, j, k]
    n[d] = c.pointStart[d]           # node index of the face plane
    ids = []
    for a in (0, 1):
        for b in (0, 1):
            q = list(n)
            t = [x for x in range(3) if x != d]
            q[t[0]] += a
            q[t[1]] += b
            ids.append(q)
    return np.mean([X[q[0] - 1, q[1] - 1, q[2] - 1] for q in ids], axis=0)


@pytest.mark.parametrize("make", [lambda: cases.cascade(**SMALL_CASCADE), lambda: cases.channel_bump(25, 17, 6),
                                  lambda: cases.cascade(**dict(cases.CASCADE_CONFIG2, nk=4))],
                         ids=["cascade", "channel", "cascade_config2_layout"])
def test_interfaces_match_node_for_node(make):
    c = make()
    conns = C.derive_connectivity(c.blocks)
    by_id = {b.id: b for b in c.blocks}
    pitch = c.meta.get("pitch")
    for b in c.blocks:
        for ic, cn in enumerate(conns[b.id]):
            if cn.BCType != 9:
                continue
            tb = by_id[cn.TargetBlock]
            tc = conns[tb.id][cn.TargetConn - 1]
            # the target of the target is this connection
            assert tc.TargetBlock == b.id and tc.TargetConn == ic + 1
            I, J, K = C.face_cells(cn)
            ib, jb, kb = C.p2p_source(cn, tc, I, J, K)
            for q in range(len(I)):
                p0 = _face_centre(b.xyz, cn, I[q], J[q], K[q])
                p1 = _face_centre(tb.xyz, tc, ib[q], jb[q], kb[q])
                d = p1 - p0
                if pitch and abs(abs(d[1]) - pitch) < 1e-9 * pitch:
                    d[1] = 0.0          # translational pitch periodicity
                if abs(d[2]) > 0 and by_id is not None and np.allclose(d[:2], 0) and "channel" in c.name:
                    d[2] = 0.0          # spanwise periodicity of the channel
                assert np.max(np.abs(d)) < 1e-9 * np.max(np.abs(p0)), (b.id, ic + 1, q, d)


def test_cascade_block_sizes():
    c = cases.cascade()
    dims = sorted(b.dims for b in c.blocks)
    assert (257, 49, 65) in dims
    assert dims.count((65, 41, 65)) == 2
    assert dims.count((121, 17, 65)) == 2


def test_cascade_config2_block_sizes():
    """The benchmark cascade: O-block 257x49x65 and passage blocks 97x33x65 as stated; the
    H-blocks take the 97 pitchwise nodes the 1-to-1 interfaces force; at least the stated
    1,507,328 interior cells."""
    c = cases.cascade(**cases.CASCADE_CONFIG2)
    dims = [b.dims for b in c.blocks]
    assert dims[0] == (257, 49, 65)
    assert dims.count((97, 33, 65)) == 2 and dims.count((65, 97, 65)) == 2
    cells = sum((a - 1) * (b - 1) * (d - 1) for a, b, d in dims)
    assert cells == 1966080 >= 1507328


def test_cascade_metrics_positive():
    c = cases.cascade(**SMALL_CASCADE)
    conns, geo = C.compute_geometry(c)
    for b in c.blocks:
        ni, nj, nk = b.dims
        v = geo[b.id]["VOL"][3:ni + 2, 3:nj + 2, 3:nk + 2]
        assert np.all(v > 0)
        d = geo[b.id]["DST"][3:ni + 2, 3:nj + 2, 3:nk + 2]
        assert np.all(d > 0)


def test_parameters_follow_parameterset():
    c = cases.channel_bump(25, 17, 6)
    p = c.params
    assert p.RXM2 == pytest.approx(0.5 * 0.5 * 1.4)
    assert p.PPF == pytest.approx(1.0 / 1.4 / 0.25)
    assert p.Rof == pytest.approx(1.2 * p.Rkf / p.Rmiuf)
    # static inflow pressure 1/(1.4 M^2) with rho = 1: the total-pressure ratio of M = 0.5
    assert p.P0in / p.PPF == pytest.approx((1 + 0.2 * 0.25) ** 3.5, rel=1e-12)


def test_square_cylinder_grid():
    """The square-cylinder O-block: positive volumes, the wrap cut and the periodic span found
    as 1-to-1 connections, the seeded velocity perturbation applied to the interior only."""
    import numpy as np
    from trans_gb300 import cases
    from trans_gb300 import case as CS
    c = cases.square_cylinder(ni=33, nj=17, nk=9)
    assert c.params.Kind_Hybrid == 3 and c.params.Kchld == 10 and c.params.Kind_Dual == 2
    conns, geo = CS.compute_geometry(c)
    g = geo[c.blocks[0].id]
    vol = g["VOL"][3:3 + 32, 3:3 + 16, 3:3 + 8]
    assert (vol > 0).all()
    st = CS.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    V = st[c.blocks[0].id]["V"]
    u = V[1][3:3 + 32, 8:3 + 16, 3:3 + 8] / V[0][3:3 + 32, 8:3 + 16, 3:3 + 8]
    assert 0.002 < np.std(u) < 0.05


def test_annular_sector_rotational_periodicity():
    """The annular sector's periodic faces carry rotateAngle = +-sector and the oracle runs it."""
    import numpy as np
    from oracle.oracle import OracleSolver
    from trans_gb300 import case as C
    from trans_gb300 import cases
    c = cases.annular_sector(ni=13, nj=9, nk=6)
    conns, geo = C.compute_geometry(c)
    angles = sorted(cn.rotateAngle for cn in conns[1] if cn.BCType == 9)
    assert np.allclose(angles, [-np.pi / 18, np.pi / 18], rtol=1e-12)
    st = C.initial_state(c, geo, Q_dst=c.meta["Q_dst"])
    o = OracleSolver(c, conns, geo, st)
    h = [o.iterate(k)[0]["DRSa"] for k in range(1, 6)]
    assert np.all(np.isfinite(h))
