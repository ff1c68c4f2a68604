// Plan and argument structures of the FP32 tile kernel (tiles.cu, batch.cu).
#pragma once

#include <cuda_runtime.h>

namespace mfem {

constexpr int kTileThreads = 256;

// Diagonal rows kept for the preconditioner pass: six (sum, compensation)
// pairs and the row's diagonal CSR position; 13 words, odd, so that the reads
// of consecutive rows by a warp hit distinct banks.
constexpr int kResStride = 13;

// One tile: rows (diagonal table), elements, off-diagonal entries and the
// contribution lists they reference.  Segment starts are 16-byte aligned and the
// *Pad counts cover whole 16-byte units, so each segment is one bulk copy.
struct TileDesc {
    int diagBegin, nRows, nRowsPad;          // into diagEnt: (row, meta, CSR position of (row, row) or -1, 0)
    int elemBegin, nElem;                    // into elems
    int offBegin, nOff, nOffPad;             // into offEnt: (pos, transposed pos or -1, meta, 0)
    int contribBegin, nContrib, nContribPad; // into contrib (u16: local elem << 4 | slot j << 2 | slot k)
    int nodeBegin, nNodes;                   // into nodes: the nodes of the tile's elements
    int mesh;                                // batch: index of the mesh the tile belongs to
};

// meta = (offset of the list in the tile's contributions) << 8 | list length

struct TilePlanView {
    const TileDesc *desc;
    const int *elems;            // element ids of each tile (ascending)
    const ushort4 *lconn;        // their nodes as indices into the tile's node list
    const int *nodes;            // each tile's nodes (0-based ids, ascending)
    const int4 *offEnt;
    const int4 *diagEnt;
    const unsigned short *contrib;
};

// Per-mesh geometry the tile kernel reads.
struct TileMesh {
    const float4 *hl;            // coordinates split into float hi + lo: hl[2n], hl[2n+1]
    const double *coord;         // FP64 coordinates (slivers)
    const int4 *e2n;             // 0-based connectivity
    const int *diagPos;
    const unsigned char *mask;   // Dirichlet bits per node, or NULL
};

// Coefficient sets of one mesh and where their results go: set s reads the
// per-element weights w + s*wStride ((B, mu) for ela, (kappa, 0) for lap, made
// by k_weights32 from the FP64 coefficients) and writes values + s*valuesStride,
// prec + s*precStride.
struct TileSets {
    const float2 *w;
    size_t wStride;
    float *values;
    size_t valuesStride;
    double *prec;                // NULL: no preconditioner
    size_t precStride;
    int nSets;
};

// Bounded-wait control of the tile kernel: the staged-copy wait gives up after
// waitLimit polls and flags MFEM_ERR_TIMEOUT; extraTx (testing only) makes the
// barrier expect bytes that never arrive, so that the limit is exercised.
struct TileCtl {
    unsigned waitLimit;
    unsigned extraTx;
    int nTiles;      // single-mesh launch: tiles in the grid
    int pfDist;      // prefetch into L2 the plan segments of tile blockIdx + pfDist (0: none)
};

// Byte offsets of the dynamic shared-memory regions.  The tile's node
// coordinates (x: hi parts, then lo parts, 32 bytes per node) and the queue of
// flagged elements (q) are needed only during phase 1; they share a region with
// the off-diagonal table and the row results, which are filled after it.
struct SmemLayout {
    int w, contrib, diag, off, res, x, q, bar, bytes;
};

SmemLayout smem_layout(int maxElem, int maxContribPad, int maxOffPad, int maxRowsPad, int maxNodes);
}  // namespace mfem
