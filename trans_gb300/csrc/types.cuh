// types.cuh -- host/device tables of the boundary gathers, sweeps and residual norms.
#pragma once
#include "dev.cuh"

namespace tg {

struct BCEntry {          // one boundary face cell of one connection (BC/Boundary.F90 dispatch)
    int kind, blk, conn, sub;
    int i, j, k, src_blk;           // face cell (node-face index along the normal)
    int s[3], l[3];                 // interior source cells (layers 0,1,2) and ghost cells (1,2,3)
    int face;                       // face cell index for SD/Grad (i + IJKAdd)
    int dir;                        // IJKDirect (1..3)
    int lor, kindsub;               // LeftOrRight, SubBCType (wall: the frame of its grid velocity)
    double cost, sint;              // interface rotation
};

struct OutletLine {       // one line of an outlet segment along j (BC/BC_Outlet.F90:50-106)
    int blk, n, first, pad_;        // entries [first, first+n) of the BC table, ascending j
};

struct SweepCell { int blk, i, j, k; };

// the sweep-order arrays of one context (element type R = the sweep arithmetic)
struct SweepView {
    const SweepCell* cells;     // cell of each sweep position
    const int* nbp;             // n x 6: positions of the lower (0..2) and upper (3..5) neighbours, -1 = none
    void* rec;                  // n x NREC records
    void* dq;                   // n x DQ_STRIDE DeltaQ
    long long n;
    void* pc;                   // n x 6 x NPC PrecondDW coefficients of the neighbours (FP64 path, IF_Precondition = 1), else null
};

// Tiled wavefront of the sweeps: the interior of every block cut into tiles of TIxTJxTK
// cells.  Tiles are numbered in a topological order of their (ti-1, tj-1, tk-1) dependencies
// (tile hyperplanes ti+tj+tk ascending); the cells of a tile are listed by the tile's own
// i+j+k planes.  Tile t owns planes plane0[t] .. plane0[t+1]-1; plane p lists the sweep
// positions item[pitem[p] .. pitem[p+1]-1]; dep[6t .. 6t+5] are the tiles holding the lower
// (0..2) and upper (3..5) neighbours, -1 = none.
struct TileView {
    int ntiles;
    const int* plane0;
    const int* pitem;
    const int* item;
    const int* dep;
};

struct NormPart {         // per-tile partial residual norms (Time/TIME_Update_V.F90:106-294)
    double sa, ma, sk, mk, so, mo;
    long long ia;                   // lexicographic index of the max of |D1/V1|
    int nan, pad_;
};

struct BlockNorms {       // per-block norms, the layout of trans_norms (include/trans_gpu.h)
    double DRSa, DUa, DRSk, DUk, DRSo, DUo;
    int Ima, Jma, Kma, nan_flag;
};

struct SweepSync {        // grid barrier state of the persistent sweep kernel
    unsigned count, gen;
    int err, pad_;
};

}  // namespace tg
