"""Wall distance on the GPU (trans_wall_distance) against the reference's brute-force loop
restated in numpy, and the whole host set-up with the device wall distance against the host
one.  Tolerance: bit-identical (the FP32 passes only choose which panels get the reference's
FP64 expression; the minimum of those is the reference's value exactly)."""
import numpy as np
import pytest

from helpers import small_cascade, small_channel
from test_walldist import brute_wall_distance, cell_centres

pytestmark = pytest.mark.gpu


def test_device_equals_brute_force(gpu_lib):
    from trans_gb300.solver import wall_distance_gpu
    for c, conns, geo, st in (small_cascade(), small_channel()):
        for xc, yc, zc in cell_centres(geo, c):
            dev = wall_distance_gpu(gpu_lib, xc, yc, zc, c.surfaces, c.params.Tiny)
            ref = brute_wall_distance(xc, yc, zc, c.surfaces, c.params.Tiny)
            assert np.array_equal(dev, ref)


def test_device_tiny_floor_and_far_points(gpu_lib):
    """Points on panel centres (DDD = 0 < tiny) and points far from every wall."""
    from trans_gb300.solver import wall_distance_gpu
    c, conns, geo, st = small_cascade()
    S0 = c.surfaces[0]
    X, Y, Z = S0[..., 0], S0[..., 1], S0[..., 2]
    xs = (X[:-1, :-1] + X[1:, :-1] + X[:-1, 1:] + X[1:, 1:]) / 4.0
    ys = (Y[:-1, :-1] + Y[1:, :-1] + Y[:-1, 1:] + Y[1:, 1:]) / 4.0
    zs = (Z[:-1, :-1] + Z[1:, :-1] + Z[:-1, 1:] + Z[1:, 1:]) / 4.0
    px = np.concatenate([xs.ravel(), [100.0, -250.0, 1.0e3]])
    py = np.concatenate([ys.ravel(), [3.0, 7.5, -1.0e3]])
    pz = np.concatenate([zs.ravel(), [0.5, 0.25, 2.0e3]])
    for surf in (c.surfaces, c.surfaces[:1]):
        dev = wall_distance_gpu(gpu_lib, px, py, pz, surf, 1.0e-20)
        ref = brute_wall_distance(px, py, pz, surf, 1.0e-20)
        assert np.array_equal(dev, ref)


def test_geometry_with_device_wall_distance_equals_host(gpu_lib):
    """The serving grid's coarse level (352 k cells, 26 k wall panels): every geometry array of
    the host set-up is bit-identical with the wall distance taken on the GPU."""
    from trans_gb300 import case as CS
    from trans_gb300 import cases
    from trans_gb300.serving import LEVELS
    from trans_gb300.solver import device_wall_distance
    c = cases.cascade(**LEVELS["coarse"])
    conns_h, geo_h = CS.compute_geometry(c)
    conns_d, geo_d = CS.compute_geometry(c, dst_fn=device_wall_distance(gpu_lib))
    for b in c.blocks:
        for name in geo_h[b.id]:
            assert np.array_equal(geo_h[b.id][name], geo_d[b.id][name]), (b.id, name)


@pytest.mark.parametrize("which", ["channel", "cascade", "cylinder", "serving_coarse"])
def test_block_metrics_on_device_equal_host(gpu_lib, which):
    """trans_block_metrics (centres, thtc, rad, Dst, SD/Grad, Alagm, boundary face centres,
    aLeng/aSeng, Vol) plus the host's corner and ghost fill-in: every geometry array of the
    set-up bit-identical to the host code."""
    from trans_gb300 import case as CS
    from trans_gb300 import cases
    from trans_gb300.serving import LEVELS
    from trans_gb300.solver import device_block_metrics
    if which == "channel":
        c = cases.channel_bump(25, 17, 6)
    elif which == "cascade":
        from helpers import SMALL_CASCADE
        c = cases.cascade(**SMALL_CASCADE)
    elif which == "cylinder":
        c = cases.square_cylinder(ni=49, nj=33, nk=9)
    else:
        c = cases.cascade(**LEVELS["coarse"])
    conns_h, geo_h = CS.compute_geometry(c)
    conns_d, geo_d = CS.compute_geometry(c, metrics_fn=device_block_metrics(gpu_lib))
    for b in c.blocks:
        assert set(geo_h[b.id]) == set(geo_d[b.id])
        for name in geo_h[b.id]:
            a, d = geo_h[b.id][name], geo_d[b.id][name]
            assert a.shape == d.shape, (b.id, name)
            assert np.array_equal(a.view(np.int64), d.view(np.int64)), (b.id, name)
