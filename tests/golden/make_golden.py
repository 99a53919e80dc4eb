"""Generate the golden vectors under tests/golden/ from the oracle.

The reference ships no tests, outputs or sample decks and cannot be built (no Fortran
compiler, no MPI), so these vectors come from the oracle (oracle/trans_oracle.cpp) run on the
seeded synthetic cases of trans_gb300/cases.py.  They pin the oracle across machines and
compilers, and the GPU tests compare the CUDA path with them; they are not an independent
check of the oracle against the reference.

    python tests/golden/make_golden.py [name ...]     (default: every case)
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from helpers import inputs_digest, small_case  # noqa: E402
from oracle.oracle import OracleSolver  # noqa: E402

NITER = 10
CASES = {
    "channel_small_mdcd_ausmpw": ("channel", dict(Kind_Spatial=3, Kind_Roe=3)),
    "channel_small_muscl_roe": ("channel", dict(Kind_Spatial=2, Kind_Roe=1)),
    "cascade_small_mdcd_ausmpw": ("cascade", dict(Kind_Spatial=3, Kind_Roe=3)),
    "channel_small_rk3_mdcd_ausmpw": ("channel", dict(Kind_Spatial=3, Kind_Roe=3, IF_RK=1, CFL_Sub_start=1.0,
                                                      CFL_Sub_end=1.0)),
    "channel_small_muscl2_roe": ("channel", dict(Kind_Spatial=1, Kind_Roe=1)),
    "cascade_small_mdcdhyb_ausmpw": ("cascade", dict(Kind_Spatial=4, Kind_Roe=3, F_limiter2=0.05)),
    "channel_small_mdcd_ausmpw_wd2006": ("channel", dict(Kind_Spatial=3, Kind_Roe=3, Kind_Model=2)),
    "cascade_small_mdcd_roerot": ("cascade", dict(Kind_Spatial=3, Kind_Roe=2)),
    "channel_small_mdcd_ausmpw_iddes": ("channel", dict(Kind_Spatial=3, Kind_Roe=3, Kind_Hybrid=3, Kind_SubHY=5)),
    "channel_small_m03_muscl_roe_precond": ("channel", dict(Kind_Spatial=2, Kind_Roe=1, IF_Precondition=1, XM=0.3)),
    "cascade_small_mdcd_ausmpw_rc": ("cascade", dict(Kind_Spatial=3, Kind_Roe=3, Kind_RotMod=1)),
    "annular_small_rotating_mdcd_roe": ("annular", dict(Kind_Spatial=3, Kind_Roe=1)),
    "annular_small_rotating_muscl_roerot": ("annular", dict(Kind_Spatial=2, Kind_Roe=2)),
}


def probe_cells(dims, n=6, seed=1):
    """Fixed interior cells (Fortran indices) spread over the block."""
    rng = np.random.default_rng(seed)
    ni, nj, nk = dims
    return [[int(rng.integers(1, ni)), int(rng.integers(1, nj)), int(rng.integers(1, nk))] for _ in range(n)]


def make_case(kind, sw):
    return small_case(kind, **sw)


def record(kind, sw):
    c, conns, geo, st = make_case(kind, sw)
    o = OracleSolver(c, conns, geo, st)
    out = {"case": kind, "switches": sw, "blocks": [list(b.dims) for b in c.blocks],
           "inputs_sha256": inputs_digest(c, geo, st)}
    # first residual, per block and component: sum and sum of squares over interior cells
    for s in ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL"):
        o.run_stage(s, 1)
    res = []
    for ib, b in enumerate(c.blocks):
        ni, nj, nk = b.dims
        D = o.get_field(ib, "D")[:, 3:ni + 2, 3:nj + 2, 3:nk + 2]
        res.append({"sum": [float(np.sum(D[q])) for q in range(7)],
                    "sumsq": [float(np.sum(D[q] ** 2)) for q in range(7)]})
    out["first_residual"] = res
    o.close()
    o = OracleSolver(c, conns, geo, st)
    hist = []
    for ki in range(1, NITER + 1):
        hist.append([n["DRSa"] for n in o.iterate(ki)])
    out["DRSa"] = hist
    probes = []
    for ib, b in enumerate(c.blocks):
        V = o.get_field(ib, "V")
        for (i, j, k) in probe_cells(b.dims, seed=ib + 1):
            probes.append({"block": ib, "at": [i, j, k], "V": [float(V[L, i + 2, j + 2, k + 2]) for L in range(7)]})
    out["probes"] = probes
    o.close()
    return out


def main():
    names = sys.argv[1:] or list(CASES)
    for name in names:
        kind, sw = CASES[name]
        g = record(kind, sw)
        g["generator"] = "tests/golden/make_golden.py (oracle, %d iterations)" % NITER
        with open(os.path.join(HERE, name + ".json"), "w") as f:
            json.dump(g, f, indent=1)
        print("wrote", name, "DRSa[0]", g["DRSa"][0][0], "DRSa[-1]", g["DRSa"][-1][0])


if __name__ == "__main__":
    main()
