"""trans_update_static_scratch: TIME_Update_V with its norm partials in the library's fixed
device buffer, against the regular update stage (trans_run_stage UPDATE), through the C ABI.

Two contexts start from the same state and run the same stages; one finishes each iteration
with the regular update, the other with the static-scratch entry point.  Two calls in a row
must give the same norms and the same updated state (tolerance 1e-11 relative, the FP64
path's bar; both run the same kernel, so they agree bit for bit in practice).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import interior, rel_err, small_channel

pytestmark = pytest.mark.gpu

TOL = 1e-11
PRE_UPDATE = ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL", "LUSGS")


def test_static_scratch_update_matches_regular_update(gpu_lib):
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_channel(Kind_Spatial=3, Kind_Roe=3)
    regular, static = Solver(c, conns, geo, st), Solver(c, conns, geo, st)
    lib = static.lib
    m = interior(c.blocks[0].dims)
    for ki in (1, 2):                       # two calls in a row
        for s in PRE_UPDATE:
            regular.run_stage(s, ki)
            static.run_stage(s, ki)
        regular.run_stage("UPDATE", ki)
        want = regular.norms()[0]
        out = (abi.TransNorms * 1)()
        rc = lib.trans_update_static_scratch(static.ctx, ki, out)
        assert rc == abi.TRANS_OK, lib.trans_last_error(static.ctx)
        got = {f: getattr(out[0], f) for f, _ in abi.TransNorms._fields_}
        for f in ("DRSa", "DUa", "DRSk", "DUk", "DRSo", "DUo"):
            assert abs(got[f] - want[f]) <= TOL * abs(want[f]), (ki, f, got[f], want[f])
        for f in ("Ima", "Jma", "Kma", "nan_flag"):
            assert got[f] == want[f], (ki, f)
        for name in ("V", "PP", "T", "RMIU"):
            err = np.max(rel_err(static.get_field(0, name), regular.get_field(0, name), m))
            assert err <= TOL, (ki, name, err)
        regular.run_stage("UPDATE_U", ki)
        static.run_stage("UPDATE_U", ki)
    regular.close()
    static.close()


def test_static_scratch_rejects_null_context(gpu_lib):
    from trans_gb300 import abi
    from trans_gb300 import native
    lib = native.load()
    assert lib.trans_update_static_scratch(None, 1, C.cast(None, C.POINTER(abi.TransNorms))) == abi.TRANS_E_ARG
