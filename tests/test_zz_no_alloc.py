"""trans_update_static_scratch: TIME_Update_V with its norm partials in the library's fixed
device buffer, against the regular update stage (trans_run_stage UPDATE), through the C ABI.

The entry point is for callers that cannot allocate device memory when they update, such as a
serving loop that has committed its whole device-memory budget to resident solves.  Two
contexts start from the same state and run the same stages; one finishes each iteration with
the regular update, the other with the static-scratch entry point.  Two calls in a row must
give the same norms and the same updated state (tolerance 1e-11 relative, the FP64 path's bar;
in the mixed path both run the same FP64 update kernel on the same FP32 increments, so the
same bar holds), and the device memory the context holds must not change across the calls;
the device's free memory must not change across the second call (the first call on a device
looks the fixed buffer up, which may load the library's device code).
An unbuilt context is refused without allocating anything.

This file is collected last on purpose, so a run that stops at its first failure has run every
other test already; it passes alone in a fresh process too.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import interior, rel_err, small_cascade, small_channel

pytestmark = pytest.mark.gpu

TOL = 1e-11
PRE_UPDATE = ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL", "LUSGS")
NORM_VALUES = ("DRSa", "DUa", "DRSk", "DUk", "DRSo", "DUo")
NORM_INDICES = ("Ima", "Jma", "Kma", "nan_flag")


def _device_free_bytes():
    import torch
    free, _ = torch.cuda.mem_get_info()
    return free


def _compare(regular, static, ki, nblk, mask_of):
    from trans_gb300 import abi
    lib = static.lib
    want = regular.norms()
    out = (abi.TransNorms * nblk)()
    held = lib.trans_device_bytes(static.ctx)
    rc = lib.trans_update_static_scratch(static.ctx, ki, out)
    assert rc == abi.TRANS_OK, lib.trans_last_error(static.ctx)
    assert lib.trans_device_bytes(static.ctx) == held, "the context's device memory changed"
    for ib in range(nblk):
        got = {f: getattr(out[ib], f) for f, _ in abi.TransNorms._fields_}
        for f in NORM_VALUES:
            assert abs(got[f] - want[ib][f]) <= TOL * abs(want[ib][f]), (ki, ib, f, got[f], want[ib][f])
        for f in NORM_INDICES:
            assert got[f] == want[ib][f], (ki, ib, f)
        for name in ("V", "PP", "T", "RMIU"):
            err = np.max(rel_err(static.get_field(ib, name), regular.get_field(ib, name), mask_of(ib)))
            assert err <= TOL, (ki, ib, name, err)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("which", ["channel", "cascade"])
def test_static_scratch_update_matches_regular_update(gpu_lib, precision, which):
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    make = small_channel if which == "channel" else small_cascade
    c, conns, geo, st = make(Kind_Spatial=3, Kind_Roe=3)
    c.params.precision = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
    regular, static = Solver(c, conns, geo, st), Solver(c, conns, geo, st)
    nblk = len(c.blocks)
    masks = [interior(b.dims) for b in c.blocks]
    free0 = None
    for ki in (1, 2):                       # two calls in a row
        for s in PRE_UPDATE:
            regular.run_stage(s, ki)
            static.run_stage(s, ki)
        regular.run_stage("UPDATE", ki)
        _compare(regular, static, ki, nblk, lambda ib: masks[ib])
        if free0 is None:
            # the first call on the device looks the fixed buffer up, which may load the
            # library's device code (and its buffer) on the device; later calls allocate nothing
            import torch
            torch.cuda.synchronize()
            free0 = _device_free_bytes()
        regular.run_stage("UPDATE_U", ki)
        static.run_stage("UPDATE_U", ki)
    import torch
    torch.cuda.synchronize()
    assert _device_free_bytes() == free0, "device memory was allocated or freed across the second call"
    regular.close()
    static.close()


def test_static_scratch_batch_context(gpu_lib):
    """Two cases of uneven size in one batch context: the per-block norms of every case match
    the regular update's."""
    from trans_gb300 import abi
    from trans_gb300.solver import Batch
    lib = gpu_lib
    cases = [small_channel(Kind_Spatial=3, Kind_Roe=3), small_cascade(Kind_Spatial=3, Kind_Roe=3)]
    regular, static = Batch(abi.TRANS_FP64), Batch(abi.TRANS_FP64)
    ids = []
    for c, conns, geo, st in cases:
        ids.append((regular.add(c, conns, geo, st), static.add(c, conns, geo, st), len(c.blocks)))
    for ki in (1, 2):
        for s in PRE_UPDATE + ("UPDATE",):
            assert lib.trans_run_stage(regular.ctx, abi.STAGE_ID[s], ki, 1) == abi.TRANS_OK
        for s in PRE_UPDATE:
            assert lib.trans_run_stage(static.ctx, abi.STAGE_ID[s], ki, 1) == abi.TRANS_OK
        held = lib.trans_device_bytes(static.ctx)
        rc = lib.trans_update_static_scratch(static.ctx, ki, C.cast(None, C.POINTER(abi.TransNorms)))
        assert rc == abi.TRANS_OK, lib.trans_last_error(static.ctx)
        assert lib.trans_device_bytes(static.ctx) == held
        for rid, sid, nb in ids:
            a, b = (abi.TransNorms * nb)(), (abi.TransNorms * nb)()
            it = C.c_int()
            assert lib.trans_batch_case_norms(regular.ctx, rid, C.byref(it), None, a) == abi.TRANS_OK
            assert lib.trans_batch_case_norms(static.ctx, sid, C.byref(it), None, b) == abi.TRANS_OK
            for ib in range(nb):
                for f in NORM_VALUES:
                    x, y = getattr(b[ib], f), getattr(a[ib], f)
                    assert abs(x - y) <= TOL * abs(y), (ki, rid, ib, f, x, y)
        for s in ("UPDATE_U",):
            assert lib.trans_run_stage(regular.ctx, abi.STAGE_ID[s], ki, 1) == abi.TRANS_OK
            assert lib.trans_run_stage(static.ctx, abi.STAGE_ID[s], ki, 1) == abi.TRANS_OK
    regular.close()
    static.close()


def test_static_scratch_refuses_unbuilt_context(gpu_lib):
    """A batch context whose work lists are not built yet (a case was just added) would have to
    allocate them: the call returns TRANS_E_ARG and the context holds the same device memory
    afterwards; once an iteration has built it, the call works."""
    from trans_gb300 import abi
    from trans_gb300.solver import Batch
    lib = gpu_lib
    bt = Batch(abi.TRANS_FP64)
    c, conns, geo, st = small_channel(Kind_Spatial=3, Kind_Roe=3)
    bt.add(c, conns, geo, st)
    held = lib.trans_device_bytes(bt.ctx)
    rc = lib.trans_update_static_scratch(bt.ctx, 1, C.cast(None, C.POINTER(abi.TransNorms)))
    assert rc == abi.TRANS_E_ARG
    assert b"not built" in lib.trans_last_error(bt.ctx)
    assert lib.trans_device_bytes(bt.ctx) == held
    bt.iterate(1)                           # builds the context; the entry point then works
    for name in PRE_UPDATE:
        assert lib.trans_run_stage(bt.ctx, abi.STAGE_ID[name], 2, 1) == abi.TRANS_OK
    assert lib.trans_update_static_scratch(bt.ctx, 2, C.cast(None, C.POINTER(abi.TransNorms))) == abi.TRANS_OK
    bt.close()


def test_static_scratch_rejects_null_context(gpu_lib):
    from trans_gb300 import abi
    from trans_gb300 import native
    lib = native.load()
    assert lib.trans_update_static_scratch(None, 1, C.cast(None, C.POINTER(abi.TransNorms))) == abi.TRANS_E_ARG
