// The FP32 tile plan, built on the device (once per mesh and pattern).
//
// The tile kernel (tiles.cu, tile_body.cuh) reads, per tile: its rows (a run of
// consecutive rows in Morton order of the node coordinates), the elements
// incident to them, the nodes of those elements, and for each row the entries
// the tile computes with the list of (element, node j, node k) contributions of
// each.  The plan is made in five steps, all on the device but the walk of
// step 4:
//   1. Morton keys of the nodes (10 bits per axis over the bounding box) and a
//      stable radix sort of the keys with the node ids (equal keys keep the
//      ascending id): the row order, and the position of each node in it;
//   2. for every node -> element incidence entry, the latest position before
//      the node's own among the element's other nodes (-1 if none): an element
//      is new to a tile that starts at position s, at row i, exactly when its
//      entry at row i has that position below s;
//   3. for every position s, the end of the tile that the greedy rule makes
//      from s: rows while the new elements fit maxElem, at most maxRows rows;
//   4. the host follows the chain 0 -> end(0) -> end(end(0)) ... (one word per
//      tile);
//   5. one CTA per tile builds the tile's lists in shared memory: a counting
//      pass gives every tile's sizes, the host lays the segments end to end
//      (16-byte aligned, padded to whole 16-byte units, one bulk copy each),
//      and a filling pass writes them.
// The lists are those of a sequential build over the same cut: elements and
// nodes ascending, every contribution list in node -> element incidence order,
// entries in row order.  The entries a tile computes for row r: the diagonal,
// entries to rows of other tiles, and (r, c) with c a later row of the tile,
// which also gives (c, r) transposed.
#include <algorithm>
#include <climits>
#include <vector>

#include "context.h"
#include "tiles.cuh"

namespace mfem {

namespace {

constexpr int kPlanThreads = 256;
constexpr int kSortItems = 16;                                // keys per thread and radix pass
constexpr int kSortTile = kPlanThreads * kSortItems;          // keys per block
constexpr int kMaxPlanElem = 2048;                            // elements per tile the builder holds

// status bits of the counting pass
constexpr int kStLongList = 1;      // an entry with more than 255 contributions
constexpr int kStPattern = 2;       // a node pair of an element missing from a row
constexpr int kStAsymmetric = 4;    // (r, c) in the pattern without (c, r)

__device__ __forceinline__ unsigned spread3(unsigned v) {   // 10 bits -> every third bit
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Bounding box of the coordinates in two launches: every block reduces a
// grid-strided share of the nodes to part[6 * block] = (lo x, y, z, hi x, y, z),
// then one block reduces the parts (nParts of them) to box[0..5].
__device__ __forceinline__ void block_minmax6(double v[6], double *sRed /* [6][32] */) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int d = 0; d < 6; d++) {
        double x = v[d];
        for (int off = 16; off; off >>= 1) {
            const double y = __shfl_xor_sync(0xffffffffu, x, off);
            x = d < 3 ? fmin(x, y) : fmax(x, y);
        }
        if (lane == 0) sRed[d * 32 + warp] = x;
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        const int d = threadIdx.x;
        double x = sRed[d * 32];
        for (int w = 1; w < nw; w++) x = d < 3 ? fmin(x, sRed[d * 32 + w]) : fmax(x, sRed[d * 32 + w]);
        v[d] = x;
    }
}

__global__ void k_bbox_part(const double *__restrict__ coord, int N, double *__restrict__ part) {
    __shared__ double sRed[6 * 32];
    double v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
        for (int d = 0; d < 3; d++) {
            const double x = coord[3 * (size_t)i + d];
            v[d] = fmin(v[d], x);
            v[3 + d] = fmax(v[3 + d], x);
        }
    block_minmax6(v, sRed);
    if (threadIdx.x < 6) part[6 * blockIdx.x + threadIdx.x] = v[threadIdx.x];
}

__global__ void k_bbox_final(const double *__restrict__ part, int nParts, double *__restrict__ box) {
    __shared__ double sRed[6 * 32];
    double v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int b = threadIdx.x; b < nParts; b += blockDim.x)
        for (int d = 0; d < 6; d++) v[d] = d < 3 ? fmin(v[d], part[6 * b + d]) : fmax(v[d], part[6 * b + d]);
    block_minmax6(v, sRed);
    if (threadIdx.x < 6) box[threadIdx.x] = v[threadIdx.x];
}

// Morton key of every node (10 bits per axis over the box) and its id.
__global__ void k_morton(const double *__restrict__ coord, int N, const double *__restrict__ box,
                         unsigned *__restrict__ key, int *__restrict__ id) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    unsigned q[3];
    for (int d = 0; d < 3; d++) {
        const double lo = box[d], hi = box[3 + d];
        const double span = hi > lo ? hi - lo : 1.0;
        const double f = (coord[3 * (size_t)i + d] - lo) / span;
        q[d] = (unsigned)fmin(1023.0, fmax(0.0, f * 1023.0));
    }
    key[i] = spread3(q[0]) | (spread3(q[1]) << 1) | (spread3(q[2]) << 2);
    id[i] = i;
}

// Radix sort pass, step 1: the digit histogram of every block's keys, stored
// digit-major (hist[d * nBlocks + b]) so that its exclusive scan gives each
// block's first output position per digit, blocks in order.
__global__ void k_radix_hist(const unsigned *__restrict__ key, int n, int shift, int *__restrict__ hist,
                             int nBlocks) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int b0 = blockIdx.x * kSortTile;
    for (int k = 0; k < kSortItems; k++) {
        const int i = b0 + k * kPlanThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(key[i] >> shift) & 255u], 1);
    }
    __syncthreads();
    hist[threadIdx.x * nBlocks + blockIdx.x] = h[threadIdx.x];
}

// Step 2: stable scatter.  A block takes its keys in index order, 256 at a
// time; a key's rank among equal digits of the round comes from the match mask
// of its warp and the counts of the warps before it.
__global__ void k_radix_scatter(const unsigned *__restrict__ keyIn, const int *__restrict__ idIn, int n,
                                int shift, const int *__restrict__ offs, int nBlocks,
                                unsigned *__restrict__ keyOut, int *__restrict__ idOut) {
    __shared__ int next[256];          // next output position of each digit
    __shared__ int wcnt[8][256];       // per-warp digit counts of the round, then their offsets
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    next[tid] = offs[tid * nBlocks + blockIdx.x];
    const int b0 = blockIdx.x * kSortTile;
    for (int k = 0; k < kSortItems; k++) {
        for (int w = 0; w < 8; w++) wcnt[w][tid] = 0;
        __syncthreads();
        const int i = b0 + k * kPlanThreads + tid;
        const bool valid = i < n;
        const unsigned kk = valid ? keyIn[i] : 0u;
        const int d = valid ? (int)((kk >> shift) & 255u) : 256;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        int run = next[tid];
        for (int w = 0; w < 8; w++) {
            const int c = wcnt[w][tid];
            wcnt[w][tid] = run;
            run += c;
        }
        next[tid] = run;
        __syncthreads();
        if (valid) {
            const int p = wcnt[warp][d] + rank;
            keyOut[p] = kk;
            idOut[p] = idIn[i];
        }
        __syncthreads();
    }
}

__global__ void k_positions(const int *__restrict__ order, int N, int *__restrict__ pos) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < N) pos[order[i]] = i;
}

// Per incidence entry of node n (element e): the latest position before pos[n]
// among e's nodes, -1 if none.
__global__ void k_prev_pos(const int *__restrict__ ptr, const int *__restrict__ ne, const int4 *__restrict__ e2n,
                           const int *__restrict__ pos, int N, int *__restrict__ prevPos) {
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    const int pn = pos[n];
    for (int q = ptr[n], qe = ptr[n + 1]; q < qe; q++) {
        const int4 v = e2n[ne[q] >> 2];
        const int p[4] = {pos[v.x], pos[v.y], pos[v.z], pos[v.w]};
        int best = -1;
        for (int k = 0; k < 4; k++)
            if (p[k] < pn) best = max(best, p[k]);
        prevPos[q] = best;
    }
}

// The greedy tile from every start position s: end[s] = the first position
// after it, or s itself when the row at s alone has more than maxElem elements.
__global__ void k_tile_end(const int *__restrict__ order, const int *__restrict__ ptr,
                           const int *__restrict__ prevPos, int N, int maxRows, int maxElem,
                           int *__restrict__ end) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= N) return;
    int count = 0, t = s;
    for (int k = 0; k < maxRows && s + k < N; k++) {
        const int r = order[s + k];
        int add = 0;
        for (int q = ptr[r], qe = ptr[r + 1]; q < qe; q++) add += prevPos[q] < s;
        if (count + add > maxElem) break;
        count += add;
        t = s + k + 1;
    }
    end[s] = t;
}

// Ascending bitonic sort of a[0, n) in shared memory by the block (n a power of
// two).  The caller synchronises before.
__device__ void block_sort(int *a, int n) {
    for (int k = 2; k <= n; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < (n >> 1); i += blockDim.x) {
                const int lo = 2 * i - (i & (j - 1)), hi = lo + j;
                const bool up = (lo & k) == 0;
                const int x = a[lo], y = a[hi];
                if ((x > y) == up) {
                    a[lo] = y;
                    a[hi] = x;
                }
            }
            __syncthreads();
        }
}

// Exclusive prefix sum over the block of one value per thread; *total gets the
// sum.  Synchronises.
__device__ int block_scan(int v, int *total, int *sWarp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int x = v;
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    if (lane == 31) sWarp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nw ? sWarp[lane] : 0;
        for (int off = 1; off < 32; off <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, off);
            if (lane >= off) w += y;
        }
        if (lane < nw) sWarp[lane] = w;
    }
    __syncthreads();
    const int before = (warp ? sWarp[warp - 1] : 0) + x - v;
    *total = sWarp[nw - 1];
    __syncthreads();
    return before;
}

__device__ __forceinline__ int warp_excl_scan(int v, int *total) {
    const int lane = threadIdx.x & 31;
    int x = v;
    for (int off = 1; off < 32; off <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    *total = __shfl_sync(0xffffffffu, x, 31);
    return x - v;
}

// First index in a[0, n) whose value is not below x.
__device__ __forceinline__ int lower_bound(const int *a, int n, int x) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Contribution code: local element l, and the gradient slots of its nodes j and
// k as the tile kernel lays them out (slot of node j = (j + l / 2) mod 4), so
// that the kernel finds gradient j at slot index code >> 2.
__device__ __forceinline__ unsigned short contrib_code(int l, int j, int k) {
    const int r = l >> 1;
    return (unsigned short)((l << 4) | (((j + r) & 3) << 2) | ((k + r) & 3));
}

struct PlanSrc {
    const int *order, *pos;          // node at each position; position of each node
    const int *ptr, *ne;             // node -> element incidence (element << 2 | local node)
    const int *prevPos;              // per incidence entry
    const int4 *e2n;                 // 0-based connectivity
    const int *rowPtr, *col;         // the pattern, 0-based columns
    const int *tileBegin;            // first position of each tile, and N
    int N, maxElem, maxRows, capE, capN;
};

struct PlanDst {
    const TileDesc *desc;
    int *elems, *nodes;
    ushort4 *lconn;
    int4 *offEnt;
    int4 *diagEnt;
    unsigned short *contrib;
    int *counts;                     // counting pass: per tile (elements, nodes, contributions, off entries)
    int *rowTotals;                  // per position: the row's (contributions, off entries), from the counting pass
    int *status;
};

// Dynamic shared memory of the tile list kernel.
struct PlanSmem {
    int *elem, *node, *nodeU, *rowNode, *rowQ0, *rowQ1, *rowFlat, *rowC, *rowO;
    int4 *e2n;
};

__device__ PlanSmem plan_smem(unsigned char *sm, const PlanSrc &S) {
    PlanSmem P;
    P.e2n = reinterpret_cast<int4 *>(sm);
    int *p = reinterpret_cast<int *>(sm + (size_t)S.capE * 16);
    P.elem = p;       p += S.capE;
    P.node = p;       p += S.capN;
    P.nodeU = p;      p += S.capN;
    P.rowNode = p;    p += S.maxRows + 1;
    P.rowQ0 = p;      p += S.maxRows + 1;
    P.rowQ1 = p;      p += S.maxRows + 1;
    P.rowFlat = p;    p += S.maxRows + 1;
    P.rowC = p;       p += S.maxRows + 1;
    P.rowO = p;
    return P;
}

size_t plan_smem_bytes(int capE, int capN, int maxRows) {
    return (size_t)capE * 16 + ((size_t)capE + 2 * (size_t)capN + 6 * ((size_t)maxRows + 1)) * 4;
}

// One CTA per tile.  FILL = false: count the tile's elements, nodes,
// contributions and off-diagonal entries (and each row's share); FILL = true:
// write the lists at the offsets of desc.
template <bool FILL>
__global__ void __launch_bounds__(kPlanThreads)
k_tile_lists(PlanSrc S, PlanDst D) {
    extern __shared__ __align__(16) unsigned char sm[];
    __shared__ int sWarp[32], sCount, sStatus;
    const PlanSmem P = plan_smem(sm, S);
    const int t = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
    const int s = S.tileBegin[t], nR = S.tileBegin[t + 1] - s;
    if (tid == 0) {
        sCount = 0;
        sStatus = 0;
    }
    // rows and their incidence ranges, flattened
    for (int lr = tid; lr < nR; lr += blockDim.x) {
        const int r = S.order[s + lr];
        P.rowNode[lr] = r;
        P.rowQ0[lr] = S.ptr[r];
        P.rowQ1[lr] = S.ptr[r + 1];
    }
    __syncthreads();
    if (tid == 0) {
        int a = 0;
        for (int lr = 0; lr < nR; lr++) {
            P.rowFlat[lr] = a;
            a += P.rowQ1[lr] - P.rowQ0[lr];
        }
        P.rowFlat[nR] = a;
    }
    __syncthreads();
    // the elements new to the tile at each of their rows: the tile's elements
    const int flat = P.rowFlat[nR];
    for (int i = tid; i < flat; i += blockDim.x) {
        int lo = 0, hi = nR;   // the row holding flat entry i
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (P.rowFlat[mid] <= i) lo = mid;
            else hi = mid;
        }
        const int q = P.rowQ0[lo] + (i - P.rowFlat[lo]);
        if (S.prevPos[q] < s) {
            const int k = atomicAdd(&sCount, 1);
            if (k < S.capE) P.elem[k] = S.ne[q] >> 2;
        }
    }
    __syncthreads();
    const int nE = min(sCount, S.maxElem);   // the cut keeps it within maxElem
    if (tid == 0 && sCount > S.maxElem) sStatus |= kStPattern;
    for (int i = nE + tid; i < S.capE; i += blockDim.x) P.elem[i] = INT_MAX;
    __syncthreads();
    block_sort(P.elem, S.capE);
    // their connectivity, and their nodes, sorted and distinct
    for (int l = tid; l < nE; l += blockDim.x) {
        const int4 v = S.e2n[P.elem[l]];
        P.e2n[l] = v;
        P.node[4 * l] = v.x;
        P.node[4 * l + 1] = v.y;
        P.node[4 * l + 2] = v.z;
        P.node[4 * l + 3] = v.w;
    }
    for (int i = 4 * nE + tid; i < S.capN; i += blockDim.x) P.node[i] = INT_MAX;
    __syncthreads();
    block_sort(P.node, S.capN);
    int nN;
    {
        const int per = S.capN / blockDim.x, i0 = tid * per;
        int cnt = 0;
        for (int i = i0; i < i0 + per; i++) {
            const int x = P.node[i];
            cnt += x != INT_MAX && (i == 0 || x != P.node[i - 1]);
        }
        int o = block_scan(cnt, &nN, sWarp);
        for (int i = i0; i < i0 + per; i++) {
            const int x = P.node[i];
            if (x != INT_MAX && (i == 0 || x != P.node[i - 1])) P.nodeU[o++] = x;
        }
    }
    __syncthreads();
    if (FILL) {
        const TileDesc &T = D.desc[t];
        for (int l = tid; l < nE; l += blockDim.x) {
            D.elems[T.elemBegin + l] = P.elem[l];
            const int4 v = P.e2n[l];
            D.lconn[T.elemBegin + l] = make_ushort4(
                (unsigned short)lower_bound(P.nodeU, nN, v.x), (unsigned short)lower_bound(P.nodeU, nN, v.y),
                (unsigned short)lower_bound(P.nodeU, nN, v.z), (unsigned short)lower_bound(P.nodeU, nN, v.w));
        }
        for (int i = tid; i < nN; i += blockDim.x) D.nodes[T.nodeBegin + i] = P.nodeU[i];
        // each row's offsets in the tile's contributions and off-diagonal table
        if (tid == 0) {
            int c = 0, o = 0;
            for (int lr = 0; lr < nR; lr++) {
                P.rowC[lr] = c;
                P.rowO[lr] = o;
                c += D.rowTotals[2 * (s + lr)];
                o += D.rowTotals[2 * (s + lr) + 1];
            }
        }
        // padding of the segments (zeros)
        for (int i = T.nContrib + tid; i < T.nContribPad; i += blockDim.x) D.contrib[T.contribBegin + i] = 0;
        for (int i = T.nRows + tid; i < T.nRowsPad; i += blockDim.x) D.diagEnt[T.diagBegin + i] = make_int4(0, 0, -1, 0);
        __syncthreads();
    }
    // rows: one warp per row, lanes over the row's entries
    int myStatus = 0;
    for (int lr = warp; lr < nR; lr += nw) {
        const int r = P.rowNode[lr], q0 = P.rowQ0[lr], q1 = P.rowQ1[lr];
        const int b = S.rowPtr[r], len = S.rowPtr[r + 1] - b;
        int rowC = 0, rowO = 0, matched = 0;
        bool hasDiag = false;
        for (int m0 = 0; m0 < len; m0 += 32) {
            const int m = m0 + lane;
            const bool act = m < len;
            int cc = act ? S.col[b + m] : -1;
            if (act && (cc < 0 || cc >= S.N)) {
                myStatus |= kStPattern;
                cc = -1;
            }
            bool keep = false;
            int cnt = 0, pc = 0;
            if (cc >= 0) {
                pc = S.pos[cc];
                keep = cc == r || pc < s || pc >= s + nR || pc > s + lr;
                for (int q = q0; q < q1; q++) {
                    const int e = S.ne[q] >> 2;
                    const int l = lower_bound(P.elem, nE, e);
                    if (l >= nE || P.elem[l] != e) {   // every element of the row is the tile's
                        myStatus |= kStPattern;
                        continue;
                    }
                    const int4 v = P.e2n[l];
                    cnt += (v.x == cc) + (v.y == cc) + (v.z == cc) + (v.w == cc);
                }
            }
            matched += cnt;
            hasDiag |= __any_sync(0xffffffffu, act && cc == r) != 0;
            int tc, to;
            const int sc = warp_excl_scan(keep ? cnt : 0, &tc);
            const int so = warp_excl_scan(keep && cc != r ? 1 : 0, &to);
            if (!FILL) {
                if (keep && cnt > 255) myStatus |= kStLongList;
            } else if (keep) {
                const TileDesc &T = D.desc[t];
                const int start = P.rowC[lr] + rowC + sc;
                const int meta = (start << 8) | cnt;
                if (cc == r) {
                    D.diagEnt[T.diagBegin + lr] = make_int4(r, meta, b + m, 0);   // b + m: the CSR position of (r, r)
                } else {
                    int tpos = -1;
                    if (pc >= s && pc < s + nR) {   // a row of this tile: the transposed position
                        const int cb = S.rowPtr[cc], ce = S.rowPtr[cc + 1];
                        for (int mm = cb; mm < ce; mm++)
                            if (S.col[mm] == r) {
                                tpos = mm;
                                break;
                            }
                        if (tpos < 0) myStatus |= kStAsymmetric;
                    }
                    D.offEnt[T.offBegin + P.rowO[lr] + rowO + so] = make_int4(b + m, tpos, meta, 0);
                }
                int k2 = start;
                for (int q = q0; q < q1; q++) {
                    const int code = S.ne[q];
                    const int l = lower_bound(P.elem, nE, code >> 2);
                    if (l >= nE || P.elem[l] != (code >> 2)) continue;   // flagged by the counting pass
                    const int4 v = P.e2n[l];
                    const int k = v.x == cc ? 0 : v.y == cc ? 1 : v.z == cc ? 2 : v.w == cc ? 3 : -1;
                    if (k >= 0) D.contrib[T.contribBegin + k2++] = contrib_code(l, code & 3, k);
                }
            }
            rowC += tc;
            rowO += to;
        }
        for (int off = 16; off; off >>= 1) matched += __shfl_xor_sync(0xffffffffu, matched, off);
        if (lane == 0) {
            // every (element, node) pair of the row's elements is one of its entries
            if (matched != 4 * (q1 - q0)) myStatus |= kStPattern;
            if (!FILL) {
                P.rowC[lr] = rowC;
                P.rowO[lr] = rowO;
                D.rowTotals[2 * (s + lr)] = rowC;
                D.rowTotals[2 * (s + lr) + 1] = rowO;
            } else if (!hasDiag) {
                D.diagEnt[D.desc[t].diagBegin + lr] = make_int4(r, 0, -1, 0);
            }
        }
    }
    if (myStatus) atomicOr(&sStatus, myStatus);
    __syncthreads();
    if (!FILL && tid == 0) {
        int c = 0, o = 0;
        for (int lr = 0; lr < nR; lr++) {
            c += P.rowC[lr];
            o += P.rowO[lr];
        }
        D.counts[4 * t] = nE;
        D.counts[4 * t + 1] = nN;
        D.counts[4 * t + 2] = c;
        D.counts[4 * t + 3] = o;
    }
    if (tid == 0 && sStatus) atomicOr(D.status, sStatus);
}

int pow2_at_least(int x) {
    int p = 1;
    while (p < x) p <<= 1;
    return p;
}

int round_up(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace

void build_tile_plan_device(Context &c) {
    TilePlan &tp = c.tiles;
    build_incidence(c);
    const int N = c.nbNodes, E = c.nbElem;
    cudaStream_t st = c.stream;
    MFEM_REQUIRE(tp.maxElem <= kMaxPlanElem, MFEM_ERR_CAPACITY,
                 "tile plan: more than 2048 elements per tile");
    MFEM_REQUIRE(N > 0 && E > 0, MFEM_ERR_CAPACITY, "tile plan: empty mesh");

    // 1. Morton order of the nodes
    DevBuf dBox, dKey, dId, dKey2, dId2, dHist, dPos, dPrev, dEnd, dScan;
    const int nParts = (int)std::min<long long>(blocks_for(N, kPlanThreads), 4096);
    double *box = (double *)dBox.reserve(6 * sizeof(double) * (size_t)(nParts + 1));
    double *part = box + 6;
    unsigned *key = (unsigned *)dKey.reserve(sizeof(unsigned) * (size_t)N);
    unsigned *key2 = (unsigned *)dKey2.reserve(sizeof(unsigned) * (size_t)N);
    int *id = (int *)dId.reserve(sizeof(int) * (size_t)N);
    int *id2 = (int *)dId2.reserve(sizeof(int) * (size_t)N);
    k_bbox_part<<<nParts, kPlanThreads, 0, st>>>(c.coord.as<double>(), N, part);
    check_launch("k_bbox_part");
    k_bbox_final<<<1, kPlanThreads, 0, st>>>(part, nParts, box);
    check_launch("k_bbox_final");
    k_morton<<<blocks_for(N, kPlanThreads), kPlanThreads, 0, st>>>(c.coord.as<double>(), N, box, key, id);
    check_launch("k_morton");
    const int nSortBlocks = (N + kSortTile - 1) / kSortTile;
    // one more word: the scan writes its total after the last entry
    int *hist = (int *)dHist.reserve(sizeof(int) * (256 * (size_t)nSortBlocks + 1));
    int *scanTmp = (int *)dScan.reserve(sizeof(int) * scan_tmp_elems(256LL * nSortBlocks));
    for (int shift = 0; shift < 30; shift += 8) {   // 30-bit keys
        k_radix_hist<<<nSortBlocks, kPlanThreads, 0, st>>>(key, N, shift, hist, nSortBlocks);
        check_launch("k_radix_hist");
        exclusive_scan_i32(hist, hist, 256LL * nSortBlocks, scanTmp, st);
        k_radix_scatter<<<nSortBlocks, kPlanThreads, 0, st>>>(key, id, N, shift, hist, nSortBlocks, key2, id2);
        check_launch("k_radix_scatter");
        std::swap(key, key2);
        std::swap(id, id2);
    }
    const int *order = id;
    int *pos = (int *)dPos.reserve(sizeof(int) * (size_t)N);
    k_positions<<<blocks_for(N, kPlanThreads), kPlanThreads, 0, st>>>(order, N, pos);
    check_launch("k_positions");

    // 2. previous positions, 3. the tile from every start
    const int *ptr = c.nodeElemPtr.as<int>(), *ne = c.nodeElem.as<int>();
    int *prevPos = (int *)dPrev.reserve(sizeof(int) * 4 * (size_t)E);
    k_prev_pos<<<blocks_for(N, kPlanThreads), kPlanThreads, 0, st>>>(ptr, ne, c.e2n.as<int4>(), pos, N, prevPos);
    check_launch("k_prev_pos");
    int *end = (int *)dEnd.reserve(sizeof(int) * (size_t)N);
    k_tile_end<<<blocks_for(N, kPlanThreads), kPlanThreads, 0, st>>>(order, ptr, prevPos, N, tp.maxRows,
                                                                        tp.maxElem, end);
    check_launch("k_tile_end");

    // 4. the chain of tiles from position 0
    std::vector<int> hEnd(N);
    MFEM_CUDA(cudaMemcpyAsync(hEnd.data(), end, sizeof(int) * (size_t)N, cudaMemcpyDeviceToHost, st));
    MFEM_CUDA(cudaStreamSynchronize(st));
    std::vector<int> tileBegin{0};
    for (int p = 0; p < N;) {
        const int q = hEnd[p];
        MFEM_REQUIRE(q > p, MFEM_ERR_CAPACITY, "tile plan: one row touches more elements than a tile holds");
        tileBegin.push_back(q);
        p = q;
    }
    const int nTiles = (int)tileBegin.size() - 1;

    // 5. per-tile lists: counting pass
    DevBuf dBegin, dCounts, dRowTot, dStatus;
    int *tb = (int *)dBegin.reserve(sizeof(int) * (size_t)(nTiles + 1));
    MFEM_CUDA(cudaMemcpyAsync(tb, tileBegin.data(), sizeof(int) * (size_t)(nTiles + 1), cudaMemcpyHostToDevice, st));
    int *counts = (int *)dCounts.reserve(sizeof(int) * 4 * (size_t)nTiles);
    int *rowTot = (int *)dRowTot.reserve(sizeof(int) * 2 * (size_t)N);
    int *status = (int *)dStatus.reserve(sizeof(int));
    MFEM_CUDA(cudaMemsetAsync(status, 0, sizeof(int), st));
    PlanSrc S;
    S.order = order;
    S.pos = pos;
    S.ptr = ptr;
    S.ne = ne;
    S.prevPos = prevPos;
    S.e2n = c.e2n.as<int4>();
    S.rowPtr = c.rowPtr.as<int>();
    S.col = c.col.as<int>();
    S.tileBegin = tb;
    S.N = N;
    S.maxElem = tp.maxElem;
    S.maxRows = tp.maxRows;
    S.capE = pow2_at_least(tp.maxElem);
    S.capN = std::max(kPlanThreads, pow2_at_least(4 * tp.maxElem));
    PlanDst D{};
    D.counts = counts;
    D.rowTotals = rowTot;
    D.status = status;
    const size_t smem = plan_smem_bytes(S.capE, S.capN, S.maxRows);
    MFEM_REQUIRE(smem <= 200 * 1024, MFEM_ERR_CAPACITY, "tile plan: tile too large for the builder");
    MFEM_CUDA(cudaFuncSetAttribute(k_tile_lists<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    MFEM_CUDA(cudaFuncSetAttribute(k_tile_lists<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_tile_lists<false><<<nTiles, kPlanThreads, smem, st>>>(S, D);
    check_launch("k_tile_lists<count>");
    std::vector<int> hCounts(4 * (size_t)nTiles);
    int hStatus = 0;
    MFEM_CUDA(cudaMemcpyAsync(hCounts.data(), counts, sizeof(int) * hCounts.size(), cudaMemcpyDeviceToHost, st));
    MFEM_CUDA(cudaMemcpyAsync(&hStatus, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    MFEM_CUDA(cudaStreamSynchronize(st));
    MFEM_REQUIRE(!(hStatus & kStPattern), MFEM_ERR_PATTERN, "tile plan: pattern misses an element pair");
    MFEM_REQUIRE(!(hStatus & kStLongList), MFEM_ERR_CAPACITY, "tile plan: too many contributions for one entry");

    // the segments end to end
    std::vector<TileDesc> tiles(nTiles);
    long long nE = 0, nN = 0, nC = 0, nD = 0, nO = 0;
    int maxElem = 0, maxContrib = 0, maxOff = 0, maxRows = 0, maxNodes = 0;
    tp.nTileElems = tp.nUnits = tp.nContrib = 0;
    for (int t = 0; t < nTiles; t++) {
        TileDesc &T = tiles[t];
        T = TileDesc{};
        const int *k = &hCounts[4 * (size_t)t];
        T.elemBegin = (int)nE;
        T.nElem = k[0];
        T.nodeBegin = (int)nN;
        T.nNodes = k[1];
        T.contribBegin = (int)nC;
        T.nContrib = k[2];
        T.nContribPad = round_up(k[2], 8);
        T.offBegin = (int)nO;
        T.nOff = T.nOffPad = k[3];
        T.diagBegin = (int)nD;
        T.nRows = tileBegin[t + 1] - tileBegin[t];
        T.nRowsPad = round_up(T.nRows, 2);
        MFEM_REQUIRE(T.nContrib < (1 << 23), MFEM_ERR_CAPACITY, "tile plan: too many contributions for one entry");
        nE += T.nElem;
        nN += T.nNodes;
        nC += T.nContribPad;
        nO += T.nOffPad;
        nD += T.nRowsPad;
        MFEM_REQUIRE(nE < INT_MAX && nN < INT_MAX && nC < INT_MAX && nO < INT_MAX, MFEM_ERR_CAPACITY,
                     "tile plan: more than 2^31 entries");
        maxElem = std::max(maxElem, T.nElem);
        maxContrib = std::max(maxContrib, T.nContribPad);
        maxOff = std::max(maxOff, T.nOffPad);
        maxRows = std::max(maxRows, T.nRowsPad);
        maxNodes = std::max(maxNodes, T.nNodes);
        tp.nTileElems += T.nElem;
        tp.nUnits += T.nOff;
        tp.nContrib += T.nContrib;
    }
    tp.nTiles = nTiles;
    tp.layout = smem_layout(std::max(maxElem, 1), maxContrib, maxOff, maxRows, maxNodes);
    tp.planMax[0] = std::max(maxElem, 1);
    tp.planMax[1] = maxContrib;
    tp.planMax[2] = maxOff;
    tp.planMax[3] = maxRows;
    tp.planMax[4] = maxNodes;
    MFEM_REQUIRE(tp.layout.bytes <= 227 * 1024, MFEM_ERR_CAPACITY,
                 "tile plan: a tile needs more than 227 KB of shared memory");

    // filling pass
    // 16 bytes of slack: the tile kernel's L2 prefetches widen segments to 16-byte boundaries
    auto alloc = [](DevBuf &d, size_t bytes) { return d.reserve(bytes + 16); };
    TileDesc *desc = (TileDesc *)alloc(tp.desc, tiles.size() * sizeof(TileDesc));
    MFEM_CUDA(cudaMemcpyAsync(desc, tiles.data(), tiles.size() * sizeof(TileDesc), cudaMemcpyHostToDevice, st));
    D.desc = desc;
    D.elems = (int *)alloc(tp.elems, (size_t)nE * 4);
    D.lconn = (ushort4 *)alloc(tp.lconn, (size_t)nE * sizeof(ushort4));
    D.nodes = (int *)alloc(tp.nodes, (size_t)nN * 4);
    D.offEnt = (int4 *)alloc(tp.offEnt, (size_t)nO * sizeof(int4));
    D.diagEnt = (int4 *)alloc(tp.diagEnt, (size_t)nD * sizeof(int4));
    D.contrib = (unsigned short *)alloc(tp.contrib, (size_t)nC * 2);
    MFEM_CUDA(cudaMemsetAsync(status, 0, sizeof(int), st));
    k_tile_lists<true><<<nTiles, kPlanThreads, smem, st>>>(S, D);
    check_launch("k_tile_lists<fill>");
    MFEM_CUDA(cudaMemcpyAsync(&hStatus, status, sizeof(int), cudaMemcpyDeviceToHost, st));
    MFEM_CUDA(cudaStreamSynchronize(st));
    MFEM_REQUIRE(!(hStatus & kStAsymmetric), MFEM_ERR_PATTERN, "tile plan: pattern is not symmetric");
    tp.built = true;
}

}  // namespace mfem
