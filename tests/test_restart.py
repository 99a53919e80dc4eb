"""Restart files in the reference's record layout (Output/OUTPUT_SaveField.F90,
Input/Init.F90:38-51, 156-169): byte layout, round trips, and a solve resumed from a restart
file against the same solve run straight through (CPU oracle)."""
import struct

import numpy as np

from helpers import interior, small_channel
from trans_gb300 import restart
from trans_gb300.case import G, _zeros


def _coded(dims):
    """V with V(L,I,J,K) = L*1e6 + I*1e4 + J*1e2 + K on the interior."""
    ni, nj, nk = dims
    V = _zeros(ni, nj, nk, (7,))
    L, I, J, K = np.meshgrid(np.arange(1, 8), np.arange(1, ni), np.arange(1, nj), np.arange(1, nk), indexing="ij")
    V[:, G + 1:G + ni, G + 1:G + nj, G + 1:G + nk] = L * 1e6 + I * 1e4 + J * 1e2 + K
    return V


def test_record_layout(tmp_path):
    dims = (5, 4, 3)
    V = _coded(dims)
    R = V[0] * 0.5
    path = tmp_path / "b.dat"
    restart.write_block(path, 17, dims, V, R, V, V, kind_dual=2)
    raw = path.read_bytes()
    # record 1: KI framed by its 4-byte length
    assert struct.unpack("<iii", raw[:12]) == (4, 17, 4)
    n = 7 * 4 * 3 * 2 * 8
    assert struct.unpack("<i", raw[12:16])[0] == n
    vals = np.frombuffer(raw[16:16 + n], dtype="<f8")
    # K fastest, then J, then I, then the component
    assert vals[0] == 1e6 + 1e4 + 1e2 + 1 and vals[1] == 1e6 + 1e4 + 1e2 + 2
    assert vals[2] == 1e6 + 1e4 + 2 * 1e2 + 1               # J advanced after NK1 = 2 values
    assert vals[3 * 2] == 1e6 + 2 * 1e4 + 1e2 + 1           # I advanced after NJ1*NK1 = 6 values
    assert vals[4 * 3 * 2] == 2e6 + 1e4 + 1e2 + 1           # component advanced after 24 values
    assert len(raw) == 12 + 3 * (n + 8) + (4 * 3 * 2 * 8 + 8)


def test_round_trip(tmp_path):
    dims = (6, 5, 4)
    rng = np.random.default_rng(3)
    V = _coded(dims)
    m = interior(dims)
    V[:, m] += rng.standard_normal(V[:, m].shape)
    R = _zeros(*dims)
    R[m] = rng.random(R[m].shape)
    for kd in (0, 1, 2):
        for rb in (8, 4):
            path = tmp_path / f"b{kd}{rb}.dat"
            restart.write_block(path, 5, dims, V, R, V * 2, V * 3, kind_dual=kd, real_bytes=rb)
            ki, V2, R2, W0, W1 = restart.read_block(path, dims, kind_dual=kd, real_bytes=rb)
            assert ki == 5
            cast = (lambda a: a) if rb == 8 else (lambda a: a.astype(np.float32).astype(np.float64))
            np.testing.assert_array_equal(V2[:, m], cast(V[:, m]))
            np.testing.assert_array_equal(R2[m], cast(R[m]))
            assert (W0 is None) == (kd == 0) and (W1 is None) == (kd != 2)
            if kd == 2:
                np.testing.assert_array_equal(W1[:, m], cast(3 * V[:, m]))


def test_resume_matches_straight_run(tmp_path):
    """6 iterations, a restart file, 6 more: the fields match a straight 12-iteration run (p
    and T are recomputed from V on restart, as the reference does, so they differ by
    rounding)."""
    from oracle.oracle import OracleSolver
    c, conns, geo, st = small_channel(Kind_Spatial=3, Kind_Roe=3)
    o = OracleSolver(c, conns, geo, st)
    for ki in range(1, 13):
        o.iterate(ki)
    ref = {n: o.get_field(0, n) for n in ("V", "PP", "T", "RMIU")}
    o.close()
    o = OracleSolver(c, conns, geo, st)
    for ki in range(1, 7):
        o.iterate(ki)
    fields = [{n: o.get_field(0, n) for n in ("V", "RMIU", "WT0", "WT1")}]
    o.close()
    restart.save_case(str(tmp_path / "r"), c, fields, ki=7)
    ki0, st2 = restart.restart_state(str(tmp_path / "r"), c, geo)
    assert ki0 == 7
    o = OracleSolver(c, conns, geo, st2)
    for ki in range(ki0, ki0 + 6):
        o.iterate(ki)
    m = interior(c.blocks[0].dims)
    for n in ("V", "PP", "T", "RMIU"):
        a, b = o.get_field(0, n), ref[n]
        err = np.max(np.abs(a[..., m] - b[..., m])) / np.max(np.abs(b[..., m]))
        assert err < 1e-9, (n, err)
    o.close()
