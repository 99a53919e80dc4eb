"""CPU checks of the oracle (the restatement the GPU path is compared with).

The reference ships no tests, fixtures or sample decks, so the oracle is pinned by known
answers derived from the reference's formulas and by analytic invariants:
  - ALIMITER (Space/UTIL_MUSCL.F90:12-15) against an exact rational evaluation;
  - AUSMPW+ (Space/CONVECT_AUSMPW_Plus.F90:204-317) and Roe (Space/CONVECT_Roe_Original.F90:
    242-407) fluxes: consistency (equal states give the analytic Euler flux);
  - free-stream preservation: a uniform state on a curved grid with no viscous terms active
    gives a residual at round-off level;
  - the committed golden vectors under tests/golden (generated by make_golden.py).
"""
import ctypes as C
import json
import math
import os
from fractions import Fraction

import numpy as np
import pytest

from helpers import interior, small_channel
from oracle import oracle

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def lib():
    return oracle.load()


def alimiter_exact(a, b):
    fa, fb = Fraction(a), Fraction(b)
    e = Fraction(1e-7)
    num = fa * (fb * fb + 2 * e * e) + fb * (2 * fa * fa + e * e)
    den = 2 * fa * fa - fa * fb + 2 * fb * fb + 3 * e * e
    s = (1 if a >= 0 else -1) + (1 if b >= 0 else -1)
    return num / den * Fraction(1, 2) * abs(s)


@pytest.mark.parametrize("a,b", [(0.3, 0.1), (-0.2, -0.5), (0.3, -0.1), (1e-3, 2e-3), (0.0, 0.4), (5.0, 5.0)])
def test_alimiter_known_answers(lib, a, b):
    got = lib.oracle_alimiter(a, b)
    want = float(alimiter_exact(a, b))
    assert got == pytest.approx(want, rel=1e-14, abs=1e-300)


def test_alimiter_limits(lib):
    # zero for opposite signs, equal slopes return the slope, the kappa=1/3 weighting of
    # (a(b^2+2e^2)+b(2a^2+e^2))/(2a^2-ab+2b^2+3e^2) for unequal slopes
    assert lib.oracle_alimiter(0.3, -0.1) == 0.0
    assert lib.oracle_alimiter(0.7, 0.7) == pytest.approx(0.7, rel=1e-12)
    assert lib.oracle_alimiter(0.2, 0.5) == pytest.approx(0.1875, rel=1e-12)
    assert lib.oracle_alimiter(0.5, 0.2) == pytest.approx(0.25, rel=1e-12)


def muscl2_exact(a, b):
    """Space/UTIL_MUSCL.F90:21-35 in exact rational arithmetic."""
    fa, fb, e = Fraction(a), Fraction(b), Fraction(1e-6)
    s = (2 * fa * fb + e) / (fa * fa + fb * fb + e)
    return ((1 + s) * fa + (1 - s) * fb) * s / 2


@pytest.mark.parametrize("a,b", [(0.3, 0.1), (-0.2, -0.5), (0.3, -0.1), (1e-3, 2e-3), (0.0, 0.4), (5.0, 5.0)])
def test_muscl2_limiter_known_answers(lib, a, b):
    assert lib.oracle_muscl2_limiter(a, b) == pytest.approx(float(muscl2_exact(a, b)), rel=1e-13, abs=1e-300)


def test_muscl2_limiter_limits(lib):
    # equal slopes: smoothness 1, the slope itself; opposite slopes of equal size: smoothness
    # (-2a^2 + e)/(2a^2 + e), nearly -1, so the result is about -a * smooth^2 ... of the first slope
    assert lib.oracle_muscl2_limiter(0.7, 0.7) == pytest.approx(0.7, rel=1e-12)
    assert lib.oracle_muscl2_limiter(0.0, 0.0) == 0.0
    s = (-2 * 0.25 + 1e-6) / (0.5 + 1e-6)
    assert lib.oracle_muscl2_limiter(0.5, -0.5) == pytest.approx(((1 + s) * 0.5 - (1 - s) * 0.5) * s / 2, rel=1e-12)


def _flux_in(p, rho, u, v, w, T, n):
    pp = rho * T / p.RXM2
    s = np.array(n, float)
    area = math.sqrt(s @ s)
    return [pp, pp, T, T, u, u, v, v, w, w, s[0], s[1], s[2], area]


def _euler_flux(p, rho, u, v, w, T, n):
    pp = rho * T / p.RXM2
    s = np.array(n, float) / math.sqrt(np.dot(n, n))
    un = u * s[0] + v * s[1] + w * s[2]
    H = 1.4 / 0.4 * pp / rho + 0.5 * (u * u + v * v + w * w)
    return -np.array([rho * un, rho * un * u + pp * s[0], rho * un * v + pp * s[1], rho * un * w + pp * s[2], rho * un * H])


@pytest.mark.parametrize("fn", ["oracle_ausmpw", "oracle_roe"])
@pytest.mark.parametrize("state", [(1.0, 1.0, 0.0, 0.0, 1.0), (1.1, 0.3, -0.2, 0.1, 0.9), (0.9, 2.1, 0.1, 0.0, 1.2)])
def test_flux_consistency(lib, fn, state):
    c, *_ = small_channel()
    p = c.params
    n = (0.3, 0.8, -0.1)
    inp = (C.c_double * 14)(*_flux_in(p, *state, n))
    out = (C.c_double * 5)()
    getattr(lib, fn)(C.byref(p), inp, out)
    want = _euler_flux(p, *state, n)
    np.testing.assert_allclose(np.array(out[:]), want, rtol=1e-12, atol=1e-12 * np.max(np.abs(want)))


def test_mdcd_reproduces_linear_data(lib):
    """On linear data every candidate stencil is exact, so the face value is exact."""
    s6 = (C.c_double * 6)(*[0.5 + 0.25 * q for q in range(6)])
    out = (C.c_double * 2)()
    lib.oracle_mdcd(s6, 0.02, out)
    face = 0.5 + 0.25 * 2.5
    assert out[0] == pytest.approx(face, rel=1e-13)
    assert out[1] == pytest.approx(face, rel=1e-13)


def test_free_stream_preservation():
    """Uniform inviscid state: the convective residual vanishes to round-off on a curved grid."""
    from oracle.oracle import OracleSolver
    c, conns, geo, st = small_channel(Kind_Spatial=2, Kind_Roe=1, IF_Turb_org=0)
    b = c.blocks[0]
    for name in ("V", "PP", "T"):
        st[1][name][...] = 0.0
    V = st[1]["V"]
    V[0][...] = 1.0; V[1][...] = 1.0; V[4][...] = c.params.PPF / 0.4 + 0.5
    st[1]["PP"][...] = c.params.PPF
    st[1]["T"][...] = 1.0
    st[1]["WT0"][...] = V; st[1]["WT1"][...] = V
    o = OracleSolver(c, conns, geo, st)
    for s in ("SPECRAD", "GRADIENT", "RESIDUAL"):
        o.run_stage(s, 1)
    D = o.get_field(0, "D")
    m = interior(b.dims)
    flux_scale = np.max(np.abs(geo[1]["GRAD"])) * c.params.PPF
    assert np.max(np.abs(D[0][m])) < 1e-12 * flux_scale
    assert np.max(np.abs(D[1:5][:, m])) < 1e-10 * flux_scale


def test_oracle_iterates_and_residual_drops():
    from oracle.oracle import OracleSolver
    c, conns, geo, st = small_channel()
    o = OracleSolver(c, conns, geo, st)
    h = [o.iterate(k)[0]["DRSa"] for k in range(1, 31)]
    assert all(np.isfinite(h))
    assert h[-1] < h[0]


GOLDEN = sorted(f for f in os.listdir(GOLD) if f.endswith(".json")) if os.path.isdir(GOLD) else []

# The host set-up is bit-reproducible across CPUs (detmath), so the oracle reproduces the
# fixtures exactly; the tolerance only absorbs a different summation order of the norms.
GOLD_TOL = 1e-12


def golden_case(g):
    from helpers import small_case
    return small_case(g["case"], **g["switches"])


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_vectors(lib, name):
    """The oracle reproduces the committed golden vectors (tests/golden/make_golden.py)."""
    g = json.load(open(os.path.join(GOLD, name)))
    from oracle.oracle import OracleSolver
    from helpers import inputs_digest
    c, conns, geo, st = golden_case(g)
    assert inputs_digest(c, geo, st) == g["inputs_sha256"], "host set-up is not bit-reproducible"
    o = OracleSolver(c, conns, geo, st)
    for s in ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL"):
        o.run_stage(s, 1)
    for ib, b in enumerate(c.blocks):
        ni, nj, nk = b.dims
        D = o.get_field(ib, "D")[:, 3:ni + 2, 3:nj + 2, 3:nk + 2]
        ref = g["first_residual"][ib]
        scale = max(abs(x) for x in ref["sumsq"]) ** 0.5
        for q in range(7):
            assert abs(np.sum(D[q]) - ref["sum"][q]) <= GOLD_TOL * scale * D[q].size
            assert np.sum(D[q] ** 2) == pytest.approx(ref["sumsq"][q], rel=GOLD_TOL, abs=1e-300)
    o.close()
    o = OracleSolver(c, conns, geo, st)
    hist = [[n["DRSa"] for n in o.iterate(k)] for k in range(1, len(g["DRSa"]) + 1)]
    np.testing.assert_allclose(hist, g["DRSa"], rtol=GOLD_TOL)
    for p in g["probes"]:
        V = o.get_field(p["block"], "V")
        i, j, k = p["at"]
        np.testing.assert_allclose([V[L, i + 2, j + 2, k + 2] for L in range(7)], p["V"], rtol=GOLD_TOL)
