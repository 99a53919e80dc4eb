"""Wall distance (Geom/CalcDst.F90:127-164): the reference's brute-force loop restated in numpy
(the checker), the host k-d tree form against it, and the argument checks of
trans_wall_distance, which answer before any device work.  Tolerance: bit-identical."""
import ctypes as C

import numpy as np
import pytest

from helpers import G, small_cascade


def brute_wall_distance(xc, yc, zc, surfaces, tiny):
    """The reference's loop: per surface the minimum of DDD = Dx*Dx + Dy*Dy + Dz*Dz over the
    panel centres; surfaces combined in order as d = max(d, tiny); if (min < d) d = min."""
    px, py, pz = xc.ravel(), yc.ravel(), zc.ravel()
    d = np.full(px.shape, 1.0e20)
    for S in surfaces:
        X, Y, Z = S[..., 0], S[..., 1], S[..., 2]
        xs = ((X[:-1, :-1] + X[1:, :-1] + X[:-1, 1:] + X[1:, 1:]) / 4.0).ravel(order="F")
        ys = ((Y[:-1, :-1] + Y[1:, :-1] + Y[:-1, 1:] + Y[1:, 1:]) / 4.0).ravel(order="F")
        zs = ((Z[:-1, :-1] + Z[1:, :-1] + Z[:-1, 1:] + Z[1:, 1:]) / 4.0).ravel(order="F")
        a = np.full(px.shape, 1.0e20)
        for q in range(0, px.size, 256):
            dx = px[q:q + 256, None] - xs[None, :]
            dy = py[q:q + 256, None] - ys[None, :]
            dz = pz[q:q + 256, None] - zs[None, :]
            ddd = dx * dx + dy * dy + dz * dz
            a[q:q + 256] = np.minimum(a[q:q + 256], ddd.min(axis=1)) if xs.size else a[q:q + 256]
        d = np.maximum(d, tiny)
        d = np.where(a < d, a, d)
    return np.sqrt(d).reshape(xc.shape)


def cell_centres(geo, c):
    out = []
    for b in c.blocks:
        ni, nj, nk = b.dims
        sl = (slice(G + 1, G + ni), slice(G + 1, G + nj), slice(G + 1, G + nk))
        out.append(tuple(geo[b.id][n][sl] for n in ("XC", "YC", "ZC")))
    return out


def test_host_kdtree_equals_brute_force():
    from trans_gb300.case import wall_distance
    c, conns, geo, st = small_cascade()
    for xc, yc, zc in cell_centres(geo, c):
        a = wall_distance(xc, yc, zc, c.surfaces, c.params.Tiny)
        b = brute_wall_distance(xc, yc, zc, c.surfaces, c.params.Tiny)
        assert np.array_equal(a, b)


def test_tiny_floor_sequence():
    """Points on panel centres (DDD = 0 < tiny): the result follows the reference's sequence,
    not a plain minimum."""
    c, conns, geo, st = small_cascade()
    S0 = c.surfaces[0]
    X, Y, Z = S0[..., 0], S0[..., 1], S0[..., 2]
    xs = (X[:-1, :-1] + X[1:, :-1] + X[:-1, 1:] + X[1:, 1:]) / 4.0
    ys = (Y[:-1, :-1] + Y[1:, :-1] + Y[:-1, 1:] + Y[1:, 1:]) / 4.0
    zs = (Z[:-1, :-1] + Z[1:, :-1] + Z[:-1, 1:] + Z[1:, 1:]) / 4.0
    d = brute_wall_distance(xs[:3, :1], ys[:3, :1], zs[:3, :1], c.surfaces, 1.0e-20)
    # surface 0 gives 0; every later surface sees max(0, tiny) = tiny first, so a later
    # surface's minimum above tiny leaves d = tiny -> sqrt(tiny) = 1e-10
    assert np.all(d == np.sqrt(1.0e-20))
    d1 = brute_wall_distance(xs[:3, :1], ys[:3, :1], zs[:3, :1], c.surfaces[:1], 1.0e-20)
    assert np.all(d1 == 0.0)


@pytest.fixture(scope="module")
def lib():
    from trans_gb300 import native
    try:
        return native.load()
    except native.NativeUnavailable as e:
        pytest.skip(str(e))


def test_wall_distance_rejects_bad_input_before_device_work(lib):
    from trans_gb300 import abi
    pts = np.array([[0.0, np.nan, 0.0]])
    nodes = np.zeros(12)
    dims = np.array([2, 2], dtype=np.int32)
    out = np.zeros(1)
    P = C.POINTER(C.c_double)
    rc = lib.trans_wall_distance(1, pts.ctypes.data_as(P), 1, dims.ctypes.data_as(C.POINTER(C.c_int)),
                                 nodes.ctypes.data_as(P), 1e-20, out.ctypes.data_as(P))
    assert rc == abi.TRANS_E_ARG
    assert b"not finite" in lib.trans_last_error(None)
    bad = np.array([0, 2], dtype=np.int32)
    pts[0, 1] = 0.0
    rc = lib.trans_wall_distance(1, pts.ctypes.data_as(P), 1, bad.ctypes.data_as(C.POINTER(C.c_int)),
                                 nodes.ctypes.data_as(P), 1e-20, out.ctypes.data_as(P))
    assert rc == abi.TRANS_E_ARG
    assert lib.trans_wall_distance(0, None, 0, None, None, 1e-20, None) == abi.TRANS_OK


def test_block_metrics_rejects_bad_input_before_device_work(lib):
    from trans_gb300 import abi
    P = C.POINTER(C.c_double)
    nodes = np.zeros(3 * 4 * 4 * 4)
    nodes[5] = np.inf
    out = np.zeros(24 * 9 * 9 * 9)
    rc = lib.trans_block_metrics(4, 4, 4, nodes.ctypes.data_as(P), 0, None, None, 1e-20, out.ctypes.data_as(P))
    assert rc == abi.TRANS_E_ARG
    assert b"not finite" in lib.trans_last_error(None)
    rc = lib.trans_block_metrics(2, 4, 4, nodes.ctypes.data_as(P), 0, None, None, 1e-20, out.ctypes.data_as(P))
    assert rc == abi.TRANS_E_ARG
