"""Block decomposition of one case over several ranks, with the cross-rank 1-to-1 interface
exchange of the reference's parallel path (Common/PARALLEL_Funcs.F90:57-87, PARALLEL_BCs;
BC/PARALLEL_BC_P2P.F90:1-257, PARALLEL_BC_sendrecv_blk).

Blocks are independent within a sub-iteration except for the two ghost passes of
BC_Boundarys: the state pass (sweep -1) and the gradient pass (sweep 0).  The LU-SGS sweeps
stop at block faces, so there is no wavefront across blocks.  A rank holds a subset of the
blocks.  Its 1-to-1 segments whose target block sits on another rank are exchanged after its
own BC_STATE and BC_GRAD stages:

- the rank packs its side of every such segment (its interior layers, 36 words per face cell
  at sweep -1 and 18 at sweep 0, in the segment's K, J, I order);
- it sends the buffer to the partner's rank and receives the partner's buffer;
- it unpacks the partner's buffer into its ghost layers through the interface's index
  transform and rotation.

Buffers travel in FP64; the reference sends them as MPI_REAL (FP32).  `StageDriver` runs one
rank's blocks stage by stage through any library exporting the C ABI under a prefix (the CUDA
library, trans_*), with the halo exchange in between.  It needs only the library's halo
entry points and a transport:

    exchange(sends, recv_keys) -> {key: numpy buffer}

`sends` is a list of (destination rank, key, buffer) and `recv_keys` a list of (source rank,
key, words).  `torch_transport()` provides this over torch.distributed (NCCL between GPUs,
gloo on host memory).
"""
import ctypes as C
from dataclasses import dataclass, replace

import numpy as np

from . import abi


def partition_blocks(blocks, nranks):
    """Owner rank of every block id: largest blocks first, each to the least-loaded rank
    (interior cells as the load), ties to the lower rank."""
    load = [0] * nranks
    owner = {}
    for b in sorted(blocks, key=lambda b: (-int(np.prod([d - 1 for d in b.dims])), b.id)):
        r = min(range(nranks), key=lambda q: (load[q], q))
        owner[b.id] = r
        load[r] += int(np.prod([d - 1 for d in b.dims]))
    return owner


def local_case(case, owner, rank):
    """The case restricted to the blocks `rank` owns (same params; connectivity unchanged, so
    its 1-to-1 segments may point at blocks of other ranks)."""
    return replace(case, blocks=[b for b in case.blocks if owner[b.id] == rank])


@dataclass
class HaloSegment:
    ib: int            # local block index on this rank
    block: int         # block id
    iconn: int         # 1-based segment index of the block
    target: int        # target block id
    tconn: int         # its segment index
    peer: int          # rank owning the target block
    ncell: int         # face cells of the segment
    partner: abi.TransConn   # the target segment's connection (for the index transform)


def face_cells(cn):
    return int(np.prod([cn.pointEnd[q] - cn.pointStart[q] + 1 for q in range(3)]))


def halo_segments(case, conns, owner, rank):
    """The 1-to-1 segments of `rank`'s blocks whose target block sits on another rank."""
    out = []
    local = [b for b in case.blocks if owner[b.id] == rank]
    for ib, b in enumerate(local):
        for ic, cn in enumerate(conns[b.id]):
            if cn.BCType != 9 or owner[cn.TargetBlock] == rank:
                continue
            out.append(HaloSegment(ib, b.id, ic + 1, cn.TargetBlock, cn.TargetConn, owner[cn.TargetBlock], face_cells(cn),
                                   conns[cn.TargetBlock][cn.TargetConn - 1]))
    return out


WORDS = {-1: 36, 0: 18}       # per face cell (BC/PARALLEL_BC_P2P.F90:73-77)


class HaloExchange:
    """Packs, exchanges and unpacks the cross-rank segments of one rank through a library's
    <prefix>halo_pack / <prefix>halo_unpack entry points."""

    def __init__(self, lib, prefix, ctx, segments, transport):
        self.lib, self.pre, self.ctx = lib, prefix, ctx
        self.segments = segments
        self.transport = transport
        self._pack = getattr(lib, prefix + "halo_pack")
        self._unpack = getattr(lib, prefix + "halo_unpack")
        dp = C.POINTER(C.c_double)
        self._pack.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, dp]
        self._unpack.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(abi.TransConn), dp]
        self.words_moved = 0

    def pack_all(self, sweep):
        """This rank's send buffers of one pass and the receives it expects: (sends, recvs) in
        the transport's form."""
        w = WORDS[sweep]
        sends, recvs = [], []
        for sg in self.segments:
            buf = np.zeros(sg.ncell * w)
            rc = self._pack(self.ctx, sweep, sg.ib, sg.iconn, buf.ctypes.data_as(C.POINTER(C.c_double)))
            if rc != 0:
                raise RuntimeError(f"halo_pack failed ({rc}) block {sg.block} segment {sg.iconn}")
            # the partner receives it for its segment (target, tconn); keys name the receiver's segment
            sends.append((sg.peer, (sg.target, sg.tconn, sweep), buf))
            recvs.append((sg.peer, (sg.block, sg.iconn, sweep), face_cells(sg.partner) * w))
        return sends, recvs

    def exchange(self, sweep):
        sends, recvs = self.pack_all(sweep)
        return self.unpack_all(sweep, self.transport(sends, recvs))

    def unpack_all(self, sweep, got):
        """Unpack the received buffers of one pass ({key: buffer}, keys as pack_all names them)."""
        for sg in self.segments:
            buf = np.ascontiguousarray(got[(sg.block, sg.iconn, sweep)], dtype=np.float64)
            partner = abi.TransConn()
            C.memmove(C.addressof(partner), C.addressof(sg.partner), C.sizeof(partner))
            rc = self._unpack(self.ctx, sweep, sg.ib, sg.iconn, C.byref(partner), buf.ctypes.data_as(C.POINTER(C.c_double)))
            if rc != 0:
                raise RuntimeError(f"halo_unpack failed ({rc}) block {sg.block} segment {sg.iconn}")
            self.words_moved += buf.size
        return len(self.segments)


def torch_transport(group=None):
    """Point-to-point exchange over torch.distributed: every rank posts its sends and receives
    together (non-blocking), then waits for all of them.  A message's tag is the receiver's
    segment (block id, segment index) and the pass, so several segments between the same two
    ranks do not mix."""
    import torch
    import torch.distributed as dist

    def tag(key):
        block, iconn, sweep = key
        return (block * 1000 + iconn) * 2 + (1 if sweep == -1 else 0)

    def run(sends, recvs):
        reqs, out = [], {}
        for peer, key, buf in sends:
            reqs.append(dist.isend(torch.from_numpy(buf), dst=peer, group=group, tag=tag(key)))
        for peer, key, words in recvs:
            t = torch.empty(words, dtype=torch.float64)
            out[key] = t
            reqs.append(dist.irecv(t, src=peer, group=group, tag=tag(key)))
        for r in reqs:
            r.wait()
        return {k: v.numpy() for k, v in out.items()}
    return run


STAGES = ("SPECRAD", "BC_STATE", "GRADIENT", "BC_GRAD", "RESIDUAL", "LUSGS", "UPDATE")


class StageDriver:
    """One rank's share of the iteration of main.F90:54-197 for a block-decomposed case: every
    stage over the rank's blocks through the C ABI, the cross-rank interface exchange after
    BC_STATE (sweep -1) and BC_GRAD (sweep 0), as PARALLEL_BCs follows BC_Boundarys in the
    reference (main.F90:72-85)."""

    def __init__(self, solver, exchange):
        self.s = solver
        self.x = exchange

    def iterate(self, ki):
        p = self.s.params
        nsub = 3 if p.IF_RK == 1 else (p.Kchld if p.Kind_Dual != 0 else 1)
        for itr in range(1, nsub + 1):
            for st in STAGES:
                self.s.run_stage(st, ki, itr)
                if st == "BC_STATE":
                    self.x.exchange(-1)
                elif st == "BC_GRAD":
                    self.x.exchange(0)
        self.s.run_stage("UPDATE_U", ki, nsub)
        return self.s.norms()
