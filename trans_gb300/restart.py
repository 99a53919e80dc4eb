"""Restart files in the reference's layout, for checkpoint and resume of a solve.

The reference writes one file per block (Output/OUTPUT_SaveField.F90:14-31) as Fortran
unformatted sequential records and reads it back at start-up when KR = 1
(Input/Init.F90:38-51):

    record 1   KI                                      default INTEGER (4 bytes)
    record 2   ((((V(LL,I,J,K),K=1,NK1),J=1,NJ1),I=1,NI1),LL=1,ML)     ML = 7
    record 3   (((Rmiu(I,J,K),K=1,NK1),J=1,NJ1),I=1,NI1)
    record 4   Wt0, as V                               if Kind_dual = 1 or 2
    record 5   Wt1, as V                               if Kind_dual = 2

K varies fastest, then J, I and the component.  Each record is framed by its byte length as a
4-byte integer before and after (the sequential-access convention of gfortran and ifort; a
record of 2 GiB or more is refused).  REAL is 8 bytes in the FP64 build of the reference
(`real_bytes=8`) and 4 bytes as shipped (`real_bytes=4`).

After reading, the reference recomputes p and T from V (Input/Init.F90:156-169) and, for a
hybrid (DES) run, restarts the time levels from V (Input/Init.F90:54-72); `restart_state`
does the same and returns the state dictionary the solvers take (trans_gb300.case.initial_state
layout: full-extent -2..N+2 arrays, ghosts zero).
"""
import struct

import numpy as np

from .case import G, _zeros

ML = 7


def _record(f, payload: bytes):
    n = len(payload)
    if n >= 2 ** 31:
        raise ValueError(f"record of {n} bytes: records of 2 GiB or more are not supported")
    f.write(struct.pack("<i", n))
    f.write(payload)
    f.write(struct.pack("<i", n))


def _read_record(f):
    head = f.read(4)
    if len(head) < 4:
        raise EOFError("missing record")
    n, = struct.unpack("<i", head)
    if n < 0:
        raise ValueError("continued (split) records are not supported")
    payload = f.read(n)
    tail = f.read(4)
    if len(payload) != n or len(tail) != 4 or struct.unpack("<i", tail)[0] != n:
        raise ValueError("corrupt record: length markers do not match")
    return payload


def _interior(a, dims, comps):
    """(comps..., NI1, NJ1, NK1) view of the interior of a full-extent array."""
    ni, nj, nk = dims
    sl = (slice(None),) * comps + (slice(G + 1, G + ni), slice(G + 1, G + nj), slice(G + 1, G + nk))
    return a[sl]


def write_block(path, ki, dims, V, Rmiu, Wt0=None, Wt1=None, kind_dual=2, real_bytes=8):
    """One block's restart file (Output/OUTPUT_SaveField.F90:21-29).  V, Wt0, Wt1: (7, NI+5,
    NJ+5, NK+5) full-extent arrays; Rmiu: (NI+5, NJ+5, NK+5)."""
    dt = np.dtype("<f8" if real_bytes == 8 else "<f4")
    with open(path, "wb") as f:
        _record(f, struct.pack("<i", int(ki)))
        _record(f, np.ascontiguousarray(_interior(V, dims, 1), dtype=dt).tobytes())
        _record(f, np.ascontiguousarray(_interior(Rmiu, dims, 0), dtype=dt).tobytes())
        if kind_dual in (1, 2):
            if Wt0 is None:
                raise ValueError("Kind_dual >= 1 writes Wt0")
            _record(f, np.ascontiguousarray(_interior(Wt0, dims, 1), dtype=dt).tobytes())
        if kind_dual == 2:
            if Wt1 is None:
                raise ValueError("Kind_dual = 2 writes Wt1")
            _record(f, np.ascontiguousarray(_interior(Wt1, dims, 1), dtype=dt).tobytes())


def read_block(path, dims, kind_dual=2, real_bytes=8):
    """Read one block's restart file (Input/Init.F90:46-51).  Returns (KI_ini, V, Rmiu, Wt0,
    Wt1) with full-extent arrays (ghosts zero); Wt0/Wt1 are None where the file has none."""
    ni, nj, nk = dims
    dt = np.dtype("<f8" if real_bytes == 8 else "<f4")
    shape = (ni - 1, nj - 1, nk - 1)

    def field(payload, comps):
        want = int(np.prod(shape)) * (ML if comps else 1) * dt.itemsize
        if len(payload) != want:
            raise ValueError(f"record of {len(payload)} bytes, expected {want} for block {dims}")
        a = np.frombuffer(payload, dtype=dt).astype(np.float64)
        full = _zeros(ni, nj, nk, (ML,) if comps else ())
        _interior(full, dims, 1 if comps else 0)[...] = a.reshape(((ML,) if comps else ()) + shape)
        return full

    with open(path, "rb") as f:
        ki, = struct.unpack("<i", _read_record(f))
        V = field(_read_record(f), True)
        Rmiu = field(_read_record(f), False)
        Wt0 = field(_read_record(f), True) if kind_dual in (1, 2) else None
        Wt1 = field(_read_record(f), True) if kind_dual == 2 else None
    return ki, V, Rmiu, Wt0, Wt1


def save_case(prefix, case, fields, ki, real_bytes=8):
    """Restart files `prefix`_blkNNN.dat of every block; `fields` per block index as returned
    by trans_gb300.solver (V, RMIU, WT0, WT1 full-extent arrays)."""
    kd = case.params.Kind_Dual
    paths = []
    for ib, b in enumerate(case.blocks):
        path = "%s_blk%03d.dat" % (prefix, b.id)
        f = fields[ib]
        write_block(path, ki, b.dims, f["V"], f["RMIU"], f.get("WT0"), f.get("WT1"), kd, real_bytes)
        paths.append(path)
    return paths


def restart_state(prefix, case, geo, real_bytes=8, kind_dual_rans=0):
    """The state after a KR = 1 start from `prefix`_blkNNN.dat (Input/Init.F90:38-72,
    156-169): V, Rmiu and the time levels from the files, p and T recomputed from V, and for a
    hybrid run the time levels restarted from V.  Returns (KI_ini, state).  The reference then
    sets the module global KI_ini to the saved value and continues at KI = KI_ini + 1
    (Input/Init.F90:37,48,92), so a CFL ramp starts over."""
    p = case.params
    kd = p.Kind_Dual
    st, kis = {}, set()
    for b in case.blocks:
        ni, nj, nk = b.dims
        ki, V, Rmiu, Wt0, Wt1 = read_block("%s_blk%03d.dat" % (prefix, b.id), b.dims, kd, real_bytes)
        kis.add(ki)
        if Wt0 is None:
            Wt0 = V.copy(order="F")
        if Wt1 is None:
            Wt1 = Wt0.copy(order="F")
        c0 = (slice(G + 1, G + ni), slice(G + 1, G + nj), slice(G + 1, G + nk))
        if p.Kind_Hybrid != 0 and kind_dual_rans == 0 and kd in (1, 2):
            Wt0[(slice(None),) + c0] = V[(slice(None),) + c0]
            if kd == 2:
                Wt1[(slice(None),) + c0] = V[(slice(None),) + c0]
        elif p.Kind_Hybrid != 0 and kind_dual_rans == 1 and kd == 2:
            Wt1[(slice(None),) + c0] = Wt0[(slice(None),) + c0]
        rad = geo[b.id]["RAD"][c0]
        om = p.omega[0]
        PP, T = _zeros(ni, nj, nk), _zeros(ni, nj, nk)
        VV = V[1][c0] * V[1][c0] + V[2][c0] * V[2][c0] + V[3][c0] * V[3][c0]
        PP[c0] = (1.4 - 1.0) * V[4][c0] - 0.5 * (1.4 - 1.0) * (VV / V[0][c0] + -((om * rad) * (om * rad)) * V[0][c0])
        T[c0] = p.RXM2 * PP[c0] / V[0][c0]
        st[b.id] = dict(V=V, PP=PP, T=T, RMIU=Rmiu, WT0=Wt0, WT1=Wt1)
    if len(kis) != 1:
        raise ValueError(f"blocks were saved at different iterations: {sorted(kis)}")
    return kis.pop(), st
