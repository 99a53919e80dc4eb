"""Field transfer through the C ABI: trans_set_fields / trans_get_fields with page-locked arrays
(transposed in place over the host link) and with pageable arrays (through the staging buffer)
against the one-array calls.  Tolerance: bit-identical (the transfers only move bits)."""
import ctypes as C

import numpy as np
import pytest

from helpers import small_cascade

pytestmark = pytest.mark.gpu

FIELDS = ("V", "PP", "T", "RMIU", "SD", "DQDXYZ", "D", "SHOCK")


def _pinned(shape):
    import torch
    n = int(np.prod(shape))
    t = torch.empty(n, dtype=torch.float64, pin_memory=True)
    return t.numpy().reshape(shape, order="F"), t


def _table(items):
    dp = C.POINTER(C.c_double)
    n = len(items)
    ib, fid, ptr = (C.c_int * n)(), (C.c_int * n)(), (dp * n)()
    for q, (b, f, a) in enumerate(items):
        ib[q], fid[q], ptr[q] = b, f, a.ctypes.data_as(dp)
    return n, ib, fid, ptr


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_get_fields_pinned_and_pageable_equal_single_calls(gpu_lib, precision):
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    c.params.precision = abi.TRANS_MIXED if precision == "mixed" else abi.TRANS_FP64
    s = Solver(c, conns, geo, st, lib=gpu_lib)
    for ki in range(1, 4):
        s.iterate(ki)
    keep, pinned, pageable, ref = [], [], [], []
    for ib, b in enumerate(c.blocks):
        for name in FIELDS:
            shape = abi.field_shape(name, *b.dims)
            a, t = _pinned(shape)
            keep.append(t)
            a[...] = np.nan
            pinned.append((ib, abi.FIELD_ID[name], a))
            pageable.append((ib, abi.FIELD_ID[name], np.full(shape, np.nan, order="F")))
            ref.append(s.get_field(ib, name, full=False))
    assert gpu_lib.trans_get_fields(s.ctx, *_table(pinned)) == 0
    assert gpu_lib.trans_get_fields(s.ctx, *_table(pageable)) == 0
    for (ib, f, a), (_, _, p), r in zip(pinned, pageable, ref):
        assert np.array_equal(a.view(np.int64), r.view(np.int64)), (ib, abi.FIELDS[f])
        assert np.array_equal(p.view(np.int64), r.view(np.int64)), (ib, abi.FIELDS[f])
    s.close()


def test_set_fields_pinned_equals_single_calls(gpu_lib):
    """A state set through page-locked arrays in one call iterates exactly like the same state
    set array by array from pageable memory."""
    from trans_gb300 import abi
    from trans_gb300.case import fortran_view
    from trans_gb300.solver import Solver, STATE_FIELDS
    c, conns, geo, st = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    rng = np.random.default_rng(5)
    for b in c.blocks:
        st[b.id]["V"][...] *= 1.0 + 1e-3 * rng.standard_normal(st[b.id]["V"].shape)
    a = Solver(c, conns, geo, st, lib=gpu_lib)            # pageable, one array per call
    c2, conns2, geo2, st2 = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    b2 = Solver(c2, conns2, geo2, st2, lib=gpu_lib)
    keep, items = [], []
    for ib, b in enumerate(c.blocks):
        for name in STATE_FIELDS:
            f = fortran_view(name, st[b.id][name])
            p, t = _pinned(f.shape)
            keep.append(t)
            p[...] = f
            items.append((ib, abi.FIELD_ID[name], p))
    assert gpu_lib.trans_set_fields(b2.ctx, *_table(items)) == 0
    for ki in range(1, 4):
        na, nb = a.iterate(ki), b2.iterate(ki)
        assert [x["DRSa"] for x in na] == [x["DRSa"] for x in nb]
    for ib in range(len(c.blocks)):
        for name in ("V", "PP", "T", "RMIU"):
            x, y = a.get_field(ib, name), b2.get_field(ib, name)
            assert np.array_equal(x.view(np.int64), y.view(np.int64)), (ib, name)
    a.close()
    b2.close()


def test_fields_reject_bad_entries(gpu_lib):
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_cascade()
    s = Solver(c, conns, geo, st, lib=gpu_lib)
    a = np.zeros(abi.field_shape("PP", *c.blocks[0].dims), order="F")
    assert gpu_lib.trans_get_fields(s.ctx, *_table([(len(c.blocks), abi.FIELD_ID["PP"], a)])) == abi.TRANS_E_ARG
    assert gpu_lib.trans_get_fields(s.ctx, *_table([(0, 99, a)])) == abi.TRANS_E_ARG
    assert gpu_lib.trans_get_fields(s.ctx, 0, None, None, None) == abi.TRANS_OK
    s.close()


def test_batch_fields_match_single_case(gpu_lib):
    """trans_batch_set_fields / trans_batch_get_fields on one case of a batch context."""
    from trans_gb300 import abi
    from trans_gb300.solver import Batch
    bt = Batch(abi.TRANS_FP64, lib=gpu_lib)
    a = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    cid = bt.add(*a)
    other = bt.add(*small_cascade(Kind_Spatial=2, Kind_Roe=1))
    bt.iterate(2)
    keep, items, ref = [], [], []
    for ib, b in enumerate(a[0].blocks):
        for name in ("V", "PP", "RMIU"):
            p, t = _pinned(abi.field_shape(name, *b.dims))
            keep.append(t)
            items.append((ib, abi.FIELD_ID[name], p))
            ref.append(bt.get_field(cid, ib, name, full=False))
    assert gpu_lib.trans_batch_get_fields(bt.ctx, cid, *_table(items)) == 0
    for (ib, f, p), r in zip(items, ref):
        assert np.array_equal(p.view(np.int64), r.view(np.int64)), (ib, abi.FIELDS[f])
    # write the same arrays back through the batch call and read them one by one
    assert gpu_lib.trans_batch_set_fields(bt.ctx, cid, *_table(items)) == 0
    for (ib, f, p), r in zip(items, ref):
        back = bt.get_field(cid, ib, abi.FIELDS[f], full=False)
        assert np.array_equal(back.view(np.int64), r.view(np.int64)), (ib, abi.FIELDS[f])
    assert gpu_lib.trans_batch_get_fields(bt.ctx, 12345, *_table(items[:1])) == abi.TRANS_E_ARG
    assert bt.norms(other)[0] == 2
    bt.close()


def test_batched_transfers_keep_call_order(gpu_lib):
    """Page-locked arrays go over the host link in batches (one launch for up to 60 arrays): a
    call with more arrays than one batch holds, and one that names the same block and field
    twice (the later array wins, as with one call per array), give what one-array calls give."""
    from trans_gb300 import abi
    from trans_gb300.solver import Solver
    c, conns, geo, st = small_cascade(Kind_Spatial=3, Kind_Roe=3)
    s = Solver(c, conns, geo, st, lib=gpu_lib)
    s.iterate(1)
    keep, items, ref = [], [], []
    for rep in range(14):                          # 70 arrays: two batches
        for ib, b in enumerate(c.blocks):
            shape = abi.field_shape("PP", *b.dims)
            a, t = _pinned(shape)
            a[...] = np.nan
            keep.append(t)
            items.append((ib, abi.FIELD_ID["PP"], a))
    assert gpu_lib.trans_get_fields(s.ctx, *_table(items)) == 0
    for ib, b in enumerate(c.blocks):
        ref = s.get_field(ib, "PP")
        for (jb, _, a) in items:
            if jb == ib:
                assert np.array_equal(a.view(np.int64), ref.view(np.int64))
    # the same block and field twice in one upload: the second array is what the slots hold
    shape = abi.field_shape("T", *c.blocks[0].dims)
    first, t1 = _pinned(shape)
    second, t2 = _pinned(shape)
    first[...] = 1.0
    second[...] = 2.0
    keep += [t1, t2]
    assert gpu_lib.trans_set_fields(s.ctx, *_table([(0, abi.FIELD_ID["T"], first), (0, abi.FIELD_ID["T"], second)])) == 0
    assert np.all(s.get_field(0, "T") == 2.0)
    s.close()
