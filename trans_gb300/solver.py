"""Python driver over the C ABI of include/trans_gpu.h.

``Solver`` plays the role of the reference's main program (main.F90): it hands the blocks,
connectivity, geometry and initial state of a case to an implementation of the ABI, then
iterates.  The implementation is the CUDA library of this package by default; any other
library exporting the same entry points under another prefix can be driven the same way.
"""
import ctypes as C

import numpy as np

from . import abi
from .case import fortran_view, full_from_fortran, markwall_arrays

GEOMETRY_FIELDS = ("SD", "GRAD", "VOL", "ALAGM", "DST", "ALENG", "ASENG", "XC", "YC", "ZC", "RAD", "THTC")
STATE_FIELDS = ("V", "PP", "T", "RMIU", "WT0", "WT1")


class SolverError(RuntimeError):
    pass


def block_table(case, conns, keep):
    """trans_block descriptors of a case (Module_Block.F90 fields); `keep` holds the buffers
    they point to for as long as the library may read them."""
    nb = len(case.blocks)
    tb = (abi.TransBlock * nb)()
    for n, b in enumerate(case.blocks):
        ni, nj, nk = b.dims
        cl = conns[b.id]
        carr = (abi.TransConn * len(cl))(*cl)
        mw = markwall_arrays(b)
        keep += [carr, mw]
        tb[n].ni, tb[n].nj, tb[n].nk, tb[n].id = ni, nj, nk, b.id
        tb[n].nconn = len(cl)
        tb[n].conn = C.cast(carr, C.POINTER(abi.TransConn))
        for f in range(6):
            tb[n].markwall[f] = mw[f].ctypes.data_as(C.POINTER(C.c_int))
    keep.append(tb)
    return tb


def _norm_dicts(arr):
    return [{f: getattr(x, f) for f, _ in abi.TransNorms._fields_} for x in arr]


class Solver:
    def __init__(self, case, conns, geo, state, lib=None, prefix="trans_", params=None):
        if lib is None:
            from . import native
            lib = native.load()
        self.lib = lib
        self.pre = prefix
        self.case = case
        self.params = params if params is not None else case.params
        self.blocks = case.blocks
        self._conns = conns
        self._keep = []
        nb = len(self.blocks)
        tb = block_table(case, conns, self._keep)
        ctx = C.c_void_p()
        rc = self._fn("create")(C.byref(self.params), nb, tb, C.byref(ctx))
        if rc != 0:
            raise SolverError(f"{prefix}create failed ({rc}: {abi.ERRORS.get(rc, '?')})")
        self.ctx = ctx
        for n, b in enumerate(self.blocks):
            for name in GEOMETRY_FIELDS:
                self.set_field(n, name, geo[b.id][name])
            for name in STATE_FIELDS:
                self.set_field(n, name, state[b.id][name])

    def _fn(self, name):
        return getattr(self.lib, self.pre + name)

    def _check(self, rc, what):
        if rc != 0:
            msg = ""
            if self.pre == "trans_":
                m = self.lib.trans_last_error(self.ctx)
                msg = m.decode() if m else ""
            raise SolverError(f"{self.pre}{what} failed ({rc}: {abi.ERRORS.get(rc, '?')}) {msg}")

    def set_field(self, ib, name, full):
        ni, nj, nk = self.blocks[ib].dims
        f = fortran_view(name, full)
        assert f.shape == abi.field_shape(name, ni, nj, nk), (name, f.shape)
        self._check(self._fn("set_field")(self.ctx, ib, abi.FIELD_ID[name], f.ctypes.data_as(C.POINTER(C.c_double))),
                    "set_field")

    def get_field(self, ib, name, full=True):
        ni, nj, nk = self.blocks[ib].dims
        f = np.zeros(abi.field_shape(name, ni, nj, nk), order="F")
        self._check(self._fn("get_field")(self.ctx, ib, abi.FIELD_ID[name], f.ctypes.data_as(C.POINTER(C.c_double))),
                    "get_field")
        return full_from_fortran(name, f, ni, nj, nk) if full else f

    def iterate(self, ki):
        nb = len(self.blocks)
        norms = (abi.TransNorms * nb)()
        rc = self._fn("iterate")(self.ctx, ki, norms)
        if rc == abi.TRANS_E_NAN:
            raise SolverError(f"NaN in iteration {ki}")
        self._check(rc, "iterate")
        return [{f: getattr(x, f) for f, _ in abi.TransNorms._fields_} for x in norms]

    def run_stage(self, stage, ki, itr=1):
        sid = abi.STAGE_ID[stage] if isinstance(stage, str) else stage
        self._check(self._fn("run_stage")(self.ctx, sid, ki, itr), "run_stage")

    def integrals(self):
        """Integrated quantities of the current state, summed on the device (trans_get_integrals)."""
        out = abi.TransIntegrals()
        self._check(self.lib.trans_get_integrals(self.ctx, C.byref(out)), "get_integrals")
        return out.as_dict()

    def wall_cp(self, ib, iconn):
        """Cp of the wall cells of wall segment iconn (1-based) of block ib, shaped (nI, nJ, nK)
        over the segment's face index ranges (Fortran order)."""
        cn = self._conns[self.blocks[ib].id][iconn - 1]
        shape = tuple(cn.pointEnd[q] - cn.pointStart[q] + 1 for q in range(3))
        cp = np.zeros(shape, order="F")
        self._check(self.lib.trans_get_wall_cp(self.ctx, ib, iconn, cp.ctypes.data_as(C.POINTER(C.c_double))),
                    "get_wall_cp")
        return cp

    def wall_forces(self, ib, iconn):
        """Pressure and viscous force of each face of wall segment iconn (1-based) of block ib:
        an array (6, nfaces), rows pressure x, y, z and viscous x, y, z, the faces in the order
        of wall_cp (I fastest, then J, then K)."""
        cn = self._conns[self.blocks[ib].id][iconn - 1]
        n = int(np.prod([cn.pointEnd[q] - cn.pointStart[q] + 1 for q in range(3)]))
        f = np.zeros((6, n), order="F")
        self._check(self.lib.trans_get_wall_forces(self.ctx, ib, iconn, f.ctypes.data_as(C.POINTER(C.c_double))),
                    "get_wall_forces")
        return f

    def norms(self):
        nb = len(self.blocks)
        norms = (abi.TransNorms * nb)()
        self._check(self._fn("get_norms")(self.ctx, norms), "get_norms")
        return [{f: getattr(x, f) for f, _ in abi.TransNorms._fields_} for x in norms]

    def close(self):
        if getattr(self, "ctx", None):
            self._fn("destroy")(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """A batch context (trans_batch_*): independent cases added and removed while it runs,
    all advanced by the same kernel launches, admitted within a device-memory budget."""

    def __init__(self, precision=abi.TRANS_FP64, budget_bytes=0, lib=None):
        if lib is None:
            from . import native
            lib = native.load()
        self.lib = lib
        ctx = C.c_void_p()
        rc = lib.trans_batch_create(precision, int(budget_bytes), C.byref(ctx))
        if rc != 0:
            raise SolverError(f"trans_batch_create failed ({rc}: {abi.ERRORS.get(rc, '?')})")
        self.ctx = ctx
        self.precision = precision
        self.cases = {}                     # id -> (case, keep)
        self.conns = {}                     # id -> connections of the case's blocks

    def _check(self, rc, what):
        if rc != 0:
            m = self.lib.trans_last_error(self.ctx)
            raise SolverError(f"trans_batch_{what} failed ({rc}: {abi.ERRORS.get(rc, '?')}) {m.decode() if m else ''}")

    def case_bytes(self, case, conns):
        keep = []
        tb = block_table(case, conns, keep)
        p = case.params
        p.precision = self.precision
        return int(self.lib.trans_batch_case_bytes(C.byref(p), len(case.blocks), tb))

    def add(self, case, conns, geo, state):
        """Admit a case; returns its id, or None if it does not fit the budget."""
        keep = []
        tb = block_table(case, conns, keep)
        p = case.params
        p.precision = self.precision
        cid = C.c_int()
        rc = self.lib.trans_batch_add(self.ctx, C.byref(p), len(case.blocks), tb, C.byref(cid))
        if rc == abi.TRANS_E_MEMORY:
            return None
        self._check(rc, "add")
        self.cases[cid.value] = (case, keep)
        self.conns[cid.value] = conns
        for n, b in enumerate(case.blocks):
            for name in GEOMETRY_FIELDS:
                self.set_field(cid.value, n, name, geo[b.id][name])
            for name in STATE_FIELDS:
                self.set_field(cid.value, n, name, state[b.id][name])
        return cid.value

    def remove(self, cid):
        self._check(self.lib.trans_batch_remove(self.ctx, cid), "remove")
        del self.cases[cid]
        self.conns.pop(cid, None)

    def set_field(self, cid, ib, name, full):
        ni, nj, nk = self.cases[cid][0].blocks[ib].dims
        f = fortran_view(name, full)
        self._check(self.lib.trans_batch_set_field(self.ctx, cid, ib, abi.FIELD_ID[name],
                                                   f.ctypes.data_as(C.POINTER(C.c_double))), "set_field")

    def get_field(self, cid, ib, name, full=True):
        ni, nj, nk = self.cases[cid][0].blocks[ib].dims
        f = np.zeros(abi.field_shape(name, ni, nj, nk), order="F")
        self._check(self.lib.trans_batch_get_field(self.ctx, cid, ib, abi.FIELD_ID[name],
                                                   f.ctypes.data_as(C.POINTER(C.c_double))), "get_field")
        return full_from_fortran(name, f, ni, nj, nk) if full else f

    def iterate(self, n=1):
        """n iterations of every case; returns True if some case produced a NaN."""
        rc = self.lib.trans_batch_iterate(self.ctx, n)
        if rc == abi.TRANS_E_NAN:
            return True
        self._check(rc, "iterate")
        return False

    def norms(self, cid):
        """(iterations done, per-block norms of the first iteration, of the last)."""
        nb = len(self.cases[cid][0].blocks)
        first, last = (abi.TransNorms * nb)(), (abi.TransNorms * nb)()
        it = C.c_int()
        self._check(self.lib.trans_batch_case_norms(self.ctx, cid, C.byref(it), first, last), "case_norms")
        return it.value, _norm_dicts(first), _norm_dicts(last)

    def integrals(self, cid=None):
        """Integrated quantities of one case, or of every case ({id: dict}) from one launch."""
        if cid is not None:
            out = abi.TransIntegrals()
            self._check(self.lib.trans_batch_get_integrals(self.ctx, cid, C.byref(out)), "get_integrals")
            return out.as_dict()
        n = len(self.cases)
        if n == 0:
            return {}
        ids, out = (C.c_int * n)(), (abi.TransIntegrals * n)()
        m = self.lib.trans_batch_integrals(self.ctx, ids, out, n)
        if m < 0:
            self._check(m, "integrals")
        return {ids[q]: out[q].as_dict() for q in range(m)}

    def wall_cp(self, cid, ib, iconn):
        case, keep = self.cases[cid]
        cn = self.conns[cid][case.blocks[ib].id][iconn - 1]
        shape = tuple(cn.pointEnd[q] - cn.pointStart[q] + 1 for q in range(3))
        cp = np.zeros(shape, order="F")
        self._check(self.lib.trans_batch_get_wall_cp(self.ctx, cid, ib, iconn, cp.ctypes.data_as(C.POINTER(C.c_double))),
                    "get_wall_cp")
        return cp

    def bytes_in_use(self):
        return int(self.lib.trans_batch_bytes_in_use(self.ctx))

    def close(self):
        if getattr(self, "ctx", None):
            self.lib.trans_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def global_residual(norms, blocks):
    """sqrt(sum N_b DRSa_b^2 / sum N_b): the block RMS norms of TIME_Update_V aggregated."""
    num = 0.0
    den = 0
    for nrm, b in zip(norms, blocks):
        n = int(np.prod([d - 1 for d in b.dims]))
        num += n * nrm["DRSa"] ** 2
        den += n
    return float(np.sqrt(num / den))


def wall_distance_gpu(lib, xc, yc, zc, surfaces, tiny):
    """trans_wall_distance: the reference's brute-force wall distance (Geom/CalcDst.F90:127-164)
    of the points (xc, yc, zc) to the panel centres of `surfaces` (node grids (NSur, MSur, 3)),
    on the GPU; same signature and result as trans_gb300.case.wall_distance."""
    pts = np.ascontiguousarray(np.stack([xc.ravel(), yc.ravel(), zc.ravel()], axis=1), dtype=np.float64)
    dims = np.array([d for S in surfaces for d in S.shape[:2]], dtype=np.int32)
    nodes = np.concatenate([S[..., q].ravel(order="F") for S in surfaces for q in range(3)]) if surfaces else np.zeros(1)
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    out = np.zeros(pts.shape[0])
    rc = lib.trans_wall_distance(pts.shape[0], pts.ctypes.data_as(C.POINTER(C.c_double)), len(surfaces),
                                 dims.ctypes.data_as(C.POINTER(C.c_int)), nodes.ctypes.data_as(C.POINTER(C.c_double)),
                                 float(tiny), out.ctypes.data_as(C.POINTER(C.c_double)))
    if rc != 0:
        m = lib.trans_last_error(None)
        raise SolverError(f"trans_wall_distance failed ({rc}: {abi.ERRORS.get(rc, '?')}) {m.decode() if m else ''}")
    return out.reshape(xc.shape)


def device_wall_distance(lib=None):
    """A dst_fn for trans_gb300.case.compute_geometry that runs the wall distance on the GPU."""
    if lib is None:
        from . import native
        lib = native.load()
    return lambda xc, yc, zc, surfaces, tiny: wall_distance_gpu(lib, xc, yc, zc, surfaces, tiny)



_GEO_SCALARS = ("XC", "YC", "ZC", "DST", "ALENG", "ASENG", "VOL", "RAD", "THTC")


def block_metrics_gpu(lib, b, surfaces, tiny):
    """trans_block_metrics: cell centres, thtc/rad, wall distance, SD/Grad, Alagm, boundary face
    centres, aLeng/aSeng and Vol of one block (Geom/CalcDst.F90:95-521) on the GPU, as the
    arrays of trans_gb300.case.block_metrics before its corner and ghost fill-in."""
    ni, nj, nk = b.dims
    nodes = np.concatenate([np.asfortranarray(b.xyz[..., q]).ravel(order="F") for q in range(3)])
    nodes = np.ascontiguousarray(nodes, dtype=np.float64)
    dims = np.array([d for S in surfaces for d in S.shape[:2]], dtype=np.int32)
    snodes = np.concatenate([S[..., q].ravel(order="F") for S in surfaces for q in range(3)]) if surfaces else np.zeros(1)
    snodes = np.ascontiguousarray(snodes, dtype=np.float64)
    shape = (ni + 5, nj + 5, nk + 5)
    P = int(np.prod(shape))
    out = np.zeros(24 * P)
    dp = C.POINTER(C.c_double)
    rc = lib.trans_block_metrics(ni, nj, nk, nodes.ctypes.data_as(dp), len(surfaces),
                                 dims.ctypes.data_as(C.POINTER(C.c_int)), snodes.ctypes.data_as(dp), float(tiny),
                                 out.ctypes.data_as(dp))
    if rc != 0:
        m = lib.trans_last_error(None)
        msg = m.decode() if m else ""
        if "negative volume" in msg:
            raise ValueError(f"block {b.id}: negative volume")
        raise SolverError(f"trans_block_metrics failed ({rc}: {abi.ERRORS.get(rc, '?')}) {msg}")
    f = lambda q: out[q * P:(q + 1) * P].reshape(shape, order="F")
    g = {n: np.asfortranarray(f(q)) for q, n in enumerate(_GEO_SCALARS)}
    g["SD"] = np.zeros((3, 3) + shape, order="F")
    for d in range(3):
        for c in range(3):
            g["SD"][d, c] = f(9 + 3 * d + c)
    g["GRAD"] = np.zeros((3,) + shape, order="F")
    g["ALAGM"] = np.zeros((3,) + shape, order="F")
    for d in range(3):
        g["GRAD"][d] = f(18 + d)
        g["ALAGM"][d] = f(21 + d)
    return g


def device_block_metrics(lib=None):
    """A metrics_fn for trans_gb300.case.compute_geometry that runs the block metrics on the GPU."""
    if lib is None:
        from . import native
        lib = native.load()
    return lambda b, surfaces, tiny: block_metrics_gpu(lib, b, surfaces, tiny)
