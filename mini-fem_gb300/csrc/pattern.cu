// CSR pattern and assembly plans, built on the device.
//
// Replaces the reference's host-side pattern code:
//   create_nodeToNode  src/matrix.cc:55-91  (row pointers + 1-based columns in
//                      first-occurrence order, from DC-lib's node->element lists)
//   create_elemToEdge  src/matrix.cc:25-52  (16 CSR positions per element)
// and adds the inverse map used by the owner-computes gather: for every CSR
// entry, the (element, j, k) pairs that add to it, in ascending element order.
//
// Steps (all on the context stream):
//   1. node -> element incidence: count, scan, fill, per-node sort (ascending
//      element id, which is the order DC_create_nodeToElem lists them in);
//   2. row pattern: one thread per row merges the nodes of its incident
//      elements into a duplicate-free list (sorted, or in the reference's first
//      occurrence order), count pass + scan + write pass;
//   3. element -> 16 positions (binary search in sorted rows, linear otherwise);
//   4. gather plan: one thread per row walks its incident elements in ascending
//      order and appends (e, j, k) to the unit of entry (r, node_k) for every
//      node_k >= r, so every unit list comes out ascending by construction.
#include <algorithm>
#include <vector>

#include "context.h"

namespace mfem {

namespace {

constexpr int kMaxRow = 128;   // longest row (distinct neighbours incl. self)
constexpr int kThreads = 256;

enum StatusBits { kMissingEntry = 2, kBadIndex = 4 };

__global__ void k_to_zero_based(const int *__restrict__ in, int *__restrict__ out,
                                long long n, int nbNodes, int *status) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int v = in[i] - 1;
    if (v < 0 || v >= nbNodes) {
        atomicOr(status, kBadIndex);
        v = 0;
    }
    out[i] = v;
}

__global__ void k_incidence_count(const int *__restrict__ e2n, long long n4, int *deg) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n4) atomicAdd(&deg[e2n[i]], 1);
}

__global__ void k_incidence_fill(const int *__restrict__ e2n, long long n4,
                                 const int *__restrict__ ptr, int *fill, int *nodeElem) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n4) return;
    int n = e2n[i];
    int s = atomicAdd(&fill[n], 1);
    nodeElem[ptr[n] + s] = (int)i;   // e*4 + j
}

__global__ void k_incidence_sort(const int *__restrict__ ptr, int *nodeElem, int nbNodes) {
    int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= nbNodes) return;
    int b = ptr[n], e = ptr[n + 1];
    for (int i = b + 1; i < e; i++) {
        int v = nodeElem[i];
        int k = i - 1;
        while (k >= b && nodeElem[k] > v) {
            nodeElem[k + 1] = nodeElem[k];
            k--;
        }
        nodeElem[k + 1] = v;
    }
}

// Distinct neighbours of row r, in sorted or first-occurrence order.
template <int ORDER>
__device__ int row_neighbours(int r, const int *__restrict__ ptr,
                              const int *__restrict__ nodeElem,
                              const int *__restrict__ e2n, int *uniq, bool &overflow) {
    int cnt = 0;
    for (int p = ptr[r]; p < ptr[r + 1]; p++) {
        int e = nodeElem[p] >> 2;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            int c = e2n[4 * e + k];
            if (ORDER == MFEM_ORDER_REFERENCE) {
                bool found = false;
                for (int m = 0; m < cnt; m++)
                    if (uniq[m] == c) { found = true; break; }
                if (!found) {
                    if (cnt < kMaxRow) uniq[cnt++] = c;
                    else overflow = true;
                }
            } else {
                int m = cnt;
                while (m > 0 && uniq[m - 1] > c) m--;
                if (m > 0 && uniq[m - 1] == c) continue;
                if (cnt >= kMaxRow) { overflow = true; continue; }
                for (int q = cnt; q > m; q--) uniq[q] = uniq[q - 1];
                uniq[m] = c;
                cnt++;
            }
        }
    }
    return cnt;
}

// Rows longer than kMaxRow are listed in longRows (count in *nLong) and sized
// and written by k_long_row, one CTA each.
template <int ORDER>
__global__ void k_row_count(const int *__restrict__ ptr, const int *__restrict__ nodeElem,
                            const int *__restrict__ e2n, int nbNodes, int *rowLen,
                            int *longRows, int *nLong) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nbNodes) return;
    int uniq[kMaxRow];
    bool overflow = false;
    int cnt = row_neighbours<ORDER>(r, ptr, nodeElem, e2n, uniq, overflow);
    if (overflow) {
        longRows[atomicAdd(nLong, 1)] = r;
        cnt = 0;
    }
    rowLen[r] = cnt;
}

template <int ORDER>
__global__ void k_row_write(const int *__restrict__ ptr, const int *__restrict__ nodeElem,
                            const int *__restrict__ e2n, int nbNodes,
                            const int *__restrict__ rowPtr, int *col, int *diagPos) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nbNodes) return;
    int uniq[kMaxRow];
    bool overflow = false;
    int cnt = row_neighbours<ORDER>(r, ptr, nodeElem, e2n, uniq, overflow);
    if (overflow) return;   // a long row: k_long_row writes it
    int base = rowPtr[r];
    int dp = -1;
    for (int m = 0; m < cnt; m++) {
        col[base + m] = uniq[m];
        if (uniq[m] == r) dp = base + m;
    }
    diagPos[r] = dp;
}

// One CTA per long row: the row's 4 x (incident elements) candidate columns,
// with their candidate index (incident element order, then node slot), are
// sorted in shared memory (bitonic, P a power of two); the first of each run of
// equal columns is a distinct neighbour, and its candidate index is its first
// occurrence.  WRITE = false: the row length; true: the columns in sorted or
// first-occurrence order, and the diagonal position.
__device__ __forceinline__ bool pair_less(int2 a, int2 b) {
    return a.x != b.x ? a.x < b.x : a.y < b.y;
}

template <int ORDER, bool WRITE>
__global__ void k_long_row(const int *__restrict__ longRows, const int *__restrict__ ptr,
                           const int *__restrict__ nodeElem, const int *__restrict__ e2n, int P,
                           int *rowLen, const int *__restrict__ rowPtr, int *col, int *diagPos) {
    extern __shared__ int2 buf[];                       // P pairs, then P first-occurrence flags
    int *first = reinterpret_cast<int *>(buf + P);
    __shared__ int part[kThreads + 1];
    const int r = longRows[blockIdx.x];
    const int b = ptr[r], M = 4 * (ptr[r + 1] - b);    // M <= P (sized on the host)
    const int tid = threadIdx.x;
    for (int i = tid; i < P; i += kThreads) {
        buf[i] = i < M ? make_int2(e2n[4 * (nodeElem[b + (i >> 2)] >> 2) + (i & 3)], i)
                       : make_int2(0x7fffffff, 0x7fffffff);
        first[i] = 0;
    }
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < P; i += kThreads) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const int2 a = buf[i], c = buf[ixj];
                    if (pair_less(c, a) == ((i & k) == 0)) {
                        buf[i] = c;
                        buf[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    // distinct columns: the first of each run; ORDER_SORTED keeps the sorted
    // position, ORDER_REFERENCE the position of the first occurrence
    for (int i = tid; i < M; i += kThreads) {
        const bool head = i == 0 || buf[i].x != buf[i - 1].x;
        if (head) first[ORDER == MFEM_ORDER_SORTED ? i : buf[i].y] = 1;
    }
    __syncthreads();
    const int chunk = (P + kThreads - 1) / kThreads, lo = min(P, tid * chunk), hi = min(P, lo + chunk);
    int cnt = 0;
    for (int i = lo; i < hi; i++) cnt += first[i];
    part[tid] = cnt;
    __syncthreads();
    if (tid == 0) {
        int run = 0;
        for (int t = 0; t < kThreads; t++) {
            const int v = part[t];
            part[t] = run;
            run += v;
        }
        part[kThreads] = run;
        if (!WRITE) rowLen[r] = run;
    }
    __syncthreads();
    if (!WRITE) return;
    int pos = rowPtr[r] + part[tid];
    for (int i = lo; i < hi; i++) {
        if (!first[i]) continue;
        // sorted: the column at sorted position i; first occurrence: candidate i
        const int c = ORDER == MFEM_ORDER_SORTED ? buf[i].x
                                                 : e2n[4 * (nodeElem[b + (i >> 2)] >> 2) + (i & 3)];
        col[pos] = c;
        if (c == r) diagPos[r] = pos;
        pos++;
    }
}

__device__ __forceinline__ int find_pos(const int *__restrict__ col, int b, int e, int c,
                                        bool sorted) {
    if (sorted) {
        int lo = b, hi = e;
        while (lo < hi) {
            int mid = (lo + hi) >> 1;
            if (col[mid] < c) lo = mid + 1; else hi = mid;
        }
        return (lo < e && col[lo] == c) ? lo : -1;
    }
    for (int p = b; p < e; p++)
        if (col[p] == c) return p;
    return -1;
}

__global__ void k_elem_pos(const int *__restrict__ e2n, long long n4,
                           const int *__restrict__ rowPtr, const int *__restrict__ col,
                           bool sorted, int *elemPos, int *status) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;   // e*4 + j
    if (i >= n4) return;
    long long e = i >> 2;
    int r = e2n[i];
    int b = rowPtr[r], en = rowPtr[r + 1];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        int p = find_pos(col, b, en, e2n[4 * e + k], sorted);
        if (p < 0) atomicOr(status, kMissingEntry);
        elemPos[i * 4 + k] = p < 0 ? 0 : p;
    }
}

// Gather plan, pass A: number of contributions of every upper entry of row r.
__global__ void k_plan_count(const int *__restrict__ ptr, const int *__restrict__ nodeElem,
                             const int *__restrict__ e2n, const int *__restrict__ rowPtr,
                             const int *__restrict__ col, bool sorted, int nbNodes,
                             int *count, int *status) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nbNodes) return;
    int b = rowPtr[r], en = rowPtr[r + 1];
    for (int p = b; p < en; p++) count[p] = 0;
    for (int q = ptr[r]; q < ptr[r + 1]; q++) {
        int e = nodeElem[q] >> 2;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            int c = e2n[4 * e + k];
            if (c < r) continue;
            int p = find_pos(col, b, en, c, sorted);
            if (p < 0) { atomicOr(status, kMissingEntry); continue; }
            count[p]++;
        }
    }
}

// Pass B: fill the lists (ascending element id since nodeElem is sorted) and
// record the transposed position of every upper off-diagonal entry (entries of
// a caller's pattern that no element touches get an empty list: value 0).
__global__ void k_plan_fill(const int *__restrict__ ptr, const int *__restrict__ nodeElem,
                            const int *__restrict__ e2n, const int *__restrict__ rowPtr,
                            const int *__restrict__ col, bool sorted, int nbNodes,
                            const int *__restrict__ start, int *fill, unsigned *contrib,
                            int *tpos, int *status) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nbNodes) return;
    int b = rowPtr[r], en = rowPtr[r + 1];
    for (int p = b; p < en; p++) {
        fill[p] = 0;
        const int c = col[p];
        if (c > r) {
            // transposed entry (c, r); the pattern must be structurally symmetric
            const int t = find_pos(col, rowPtr[c], rowPtr[c + 1], r, sorted);
            if (t < 0) atomicOr(status, kMissingEntry);
            tpos[p] = t < 0 ? p : t;
        }
    }
    for (int q = ptr[r]; q < ptr[r + 1]; q++) {
        int ej = nodeElem[q];
        int e = ej >> 2, j = ej & 3;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            int c = e2n[4 * e + k];
            if (c < r) continue;
            int p = find_pos(col, b, en, c, sorted);
            if (p < 0) continue;
            contrib[start[p] + fill[p]] = ((unsigned)e << 4) | ((unsigned)j << 2) | (unsigned)k;
            fill[p]++;
        }
    }
}

// Units in element-locality order.  A unit's key is its first (smallest)
// contributing element, in windows of 512 elements, then its contribution count:
// the warps of a window read gradient records of nearby elements (which the L2
// keeps), and most of them loop the same number of times.  Placement within a
// key is in atomic order, which changes where a unit runs but not its sum.
constexpr int kOwnerShift = 9;
constexpr int kUnitCountBins = 16;
constexpr int kDiagCountBins = 32;

__global__ void k_unit_key(const int *__restrict__ rowOf, const int *__restrict__ col,
                           const int *__restrict__ start, const unsigned *__restrict__ contrib,
                           int nnz, int *key, int *keyCount) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nnz) return;
    if (col[p] <= rowOf[p]) {
        key[p] = -1;
        return;
    }
    const int n = start[p + 1] - start[p];
    const unsigned owner = n > 0 ? contrib[start[p]] >> 4 : 0u;
    const int k = (int)(owner >> kOwnerShift) * kUnitCountBins + min(max(n, 1) - 1, kUnitCountBins - 1);
    key[p] = k;
    atomicAdd(&keyCount[k], 1);
}

__global__ void k_unit_place(const int *__restrict__ key, const int *__restrict__ tpos, int nnz,
                             int *keyFill, int2 *unitPos) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nnz) return;
    const int k = key[p];
    if (k < 0) return;
    unitPos[atomicAdd(&keyFill[k], 1)] = make_int2(p, tpos[p]);
}

// Diagonal units (one per node) keyed the same way by the node's first
// incident element and its number of incident elements.
__global__ void k_diag_key(const int *__restrict__ ptr, const int *__restrict__ nodeElem,
                           int nbNodes, int *key, int *keyCount) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nbNodes) return;
    const int n = ptr[r + 1] - ptr[r];
    const unsigned owner = n > 0 ? (unsigned)nodeElem[ptr[r]] >> 2 : 0u;
    const int k = (int)(owner >> kOwnerShift) * kDiagCountBins + min(max(n, 1) - 1, kDiagCountBins - 1);
    key[r] = k;
    atomicAdd(&keyCount[k], 1);
}

__global__ void k_diag_place(const int *__restrict__ key, int nbNodes, int *keyFill,
                             int *diagNode) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nbNodes) return;
    diagNode[atomicAdd(&keyFill[key[r]], 1)] = r;
}

__global__ void k_row_of(const int *__restrict__ rowPtr, int nbNodes, int *rowOf) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nbNodes) return;
    for (int p = rowPtr[r]; p < rowPtr[r + 1]; p++) rowOf[p] = r;
}

void check_status(Context &c, const char *what) {
    int st = 0;
    read_status(c, &st, 1);
    if (st & kBadIndex)
        throw Error(MFEM_ERR_INVALID_ARG, std::string(what) + ": elemToNode index out of range");
    if (st & kMissingEntry)
        throw Error(MFEM_ERR_PATTERN, std::string(what) + ": pattern misses an element pair");
}

}  // namespace

void build_incidence(Context &c) {
    if (c.hasIncidence) return;
    const long long n4 = 4LL * c.nbElem;
    const int N = c.nbNodes;
    int *ptr = (int *)c.nodeElemPtr.reserve(sizeof(int) * (N + 1));
    int *deg = (int *)c.scratch.reserve(sizeof(int) * (size_t)(N + 1) * 2);
    int *fill = deg + (N + 1);
    int *tmp = (int *)c.scanTmp.reserve(sizeof(int) * scan_tmp_elems(N + 1));
    MFEM_CUDA(cudaMemsetAsync(deg, 0, sizeof(int) * (size_t)(N + 1) * 2, c.stream));
    k_incidence_count<<<blocks_for(n4, kThreads), kThreads, 0, c.stream>>>(c.e2n.as<int>(), n4, deg);
    check_launch("k_incidence_count");
    exclusive_scan_i32(deg, ptr, N, tmp, c.stream);
    int *ne = (int *)c.nodeElem.reserve(sizeof(int) * (size_t)n4);
    k_incidence_fill<<<blocks_for(n4, kThreads), kThreads, 0, c.stream>>>(c.e2n.as<int>(), n4, ptr, fill, ne);
    check_launch("k_incidence_fill");
    k_incidence_sort<<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(ptr, ne, N);
    check_launch("k_incidence_sort");
    c.hasIncidence = true;
}

namespace {

// Caller's node -> element lists (0-based element ids) -> the e*4 form the row
// kernels read (they use the element id only); ids outside [0, nbElem) are
// flagged and replaced by 0.
__global__ void k_caller_incidence(const int *__restrict__ in, int *__restrict__ out, long long n,
                                   int nbElem, int *status) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int e = in[i];
    if (e < 0 || e >= nbElem) {
        atomicOr(status, kBadIndex);
        e = 0;
    }
    out[i] = e << 2;
}

// Rows of the pattern from node -> element lists ptr/ne (any order within a
// node; the first-occurrence column order follows it).
void build_rows(Context &c, int order, const int *ptr, const int *ne) {
    const int N = c.nbNodes;
    int *st = status_ptr(c);
    MFEM_CUDA(cudaMemsetAsync(st, 0, sizeof(int), c.stream));
    int *rowPtr = (int *)c.rowPtr.reserve(sizeof(int) * (N + 1));
    int *tmp = (int *)c.scanTmp.reserve(sizeof(int) * scan_tmp_elems(N + 1));
    const int *e2n = c.e2n.as<int>();
    int *longRows = (int *)c.scratch2.reserve(sizeof(int) * ((size_t)N + 1));
    int *nLongDev = longRows + N;
    MFEM_CUDA(cudaMemsetAsync(nLongDev, 0, sizeof(int), c.stream));
    if (order == MFEM_ORDER_SORTED)
        k_row_count<MFEM_ORDER_SORTED><<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(ptr, ne, e2n, N, rowPtr, longRows, nLongDev);
    else
        k_row_count<MFEM_ORDER_REFERENCE><<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(ptr, ne, e2n, N, rowPtr, longRows, nLongDev);
    check_launch("k_row_count");
    // rows longer than the per-thread list: one CTA each, candidates sorted in
    // shared memory (P = the next power of two of 4 x the largest valence)
    int nLong = 0, P = 0;
    MFEM_CUDA(cudaMemcpyAsync(&nLong, nLongDev, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaStreamSynchronize(c.stream));
    if (nLong > 0) {
        std::vector<int> rows(nLong), hptr(N + 1);
        MFEM_CUDA(cudaMemcpyAsync(rows.data(), longRows, sizeof(int) * nLong, cudaMemcpyDeviceToHost, c.stream));
        MFEM_CUDA(cudaMemcpyAsync(hptr.data(), ptr, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, c.stream));
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
        int maxM = 0;
        for (int r : rows) maxM = std::max(maxM, 4 * (hptr[r + 1] - hptr[r]));
        P = 1;
        while (P < maxM) P <<= 1;
        MFEM_REQUIRE((size_t)P * 12 <= 200 * 1024, MFEM_ERR_CAPACITY,
                     "create_nodeToNode: a node has more than 4096 incident elements");
        const size_t smem = (size_t)P * 12;
        if (order == MFEM_ORDER_SORTED) {
            MFEM_CUDA(cudaFuncSetAttribute(k_long_row<MFEM_ORDER_SORTED, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k_long_row<MFEM_ORDER_SORTED, false><<<nLong, kThreads, smem, c.stream>>>(longRows, ptr, ne, e2n, P, rowPtr, nullptr, nullptr, nullptr);
        } else {
            MFEM_CUDA(cudaFuncSetAttribute(k_long_row<MFEM_ORDER_REFERENCE, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k_long_row<MFEM_ORDER_REFERENCE, false><<<nLong, kThreads, smem, c.stream>>>(longRows, ptr, ne, e2n, P, rowPtr, nullptr, nullptr, nullptr);
        }
        check_launch("k_long_row");
    }
    exclusive_scan_i32(rowPtr, rowPtr, N, tmp, c.stream);
    int nnz = 0;
    MFEM_CUDA(cudaMemcpyAsync(&nnz, rowPtr + N, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaStreamSynchronize(c.stream));
    check_status(c, "create_nodeToNode");
    int *col = (int *)c.col.reserve(sizeof(int) * (size_t)nnz);
    int *diag = (int *)c.diagPos.reserve(sizeof(int) * (size_t)N);
    if (order == MFEM_ORDER_SORTED)
        k_row_write<MFEM_ORDER_SORTED><<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(ptr, ne, e2n, N, rowPtr, col, diag);
    else
        k_row_write<MFEM_ORDER_REFERENCE><<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(ptr, ne, e2n, N, rowPtr, col, diag);
    check_launch("k_row_write");
    if (nLong > 0) {
        const size_t smem = (size_t)P * 12;
        if (order == MFEM_ORDER_SORTED) {
            MFEM_CUDA(cudaFuncSetAttribute(k_long_row<MFEM_ORDER_SORTED, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k_long_row<MFEM_ORDER_SORTED, true><<<nLong, kThreads, smem, c.stream>>>(longRows, ptr, ne, e2n, P, nullptr, rowPtr, col, diag);
        } else {
            MFEM_CUDA(cudaFuncSetAttribute(k_long_row<MFEM_ORDER_REFERENCE, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            k_long_row<MFEM_ORDER_REFERENCE, true><<<nLong, kThreads, smem, c.stream>>>(longRows, ptr, ne, e2n, P, nullptr, rowPtr, col, diag);
        }
        check_launch("k_long_row");
    }
    c.nnz = nnz;
    c.order = order;
    c.hasPattern = true;
    c.hasElemPos = false;
    c.gather.built = false;
    c.tiles.built = false;
}

}  // namespace

void build_pattern(Context &c, int order) {
    MFEM_REQUIRE(order == MFEM_ORDER_SORTED || order == MFEM_ORDER_REFERENCE,
                 MFEM_ERR_INVALID_ARG, "unknown column order");
    build_incidence(c);
    build_rows(c, order, c.nodeElemPtr.as<int>(), c.nodeElem.as<int>());
}

void build_pattern_from_incidence(Context &c, const int *hIndex, const int *hValue) {
    MFEM_REQUIRE(hIndex && hValue, MFEM_ERR_INVALID_ARG, "null nodeToElem");
    const int N = c.nbNodes;
    MFEM_REQUIRE(hIndex[0] == 0, MFEM_ERR_INVALID_ARG, "nodeToElem.index[0] must be 0");
    for (int i = 0; i < N; i++)
        MFEM_REQUIRE(hIndex[i + 1] >= hIndex[i], MFEM_ERR_INVALID_ARG,
                     "nodeToElem.index must be non-decreasing");
    const long long total = hIndex[N];
    MFEM_REQUIRE(total <= 64LL * c.nbElem, MFEM_ERR_INVALID_ARG,
                 "nodeToElem lists more incidences than the mesh can have");
    DevBuf dptr, dne, raw;
    int *ptr = (int *)dptr.reserve(sizeof(int) * ((size_t)N + 1));
    int *ne = (int *)dne.reserve(sizeof(int) * (size_t)std::max(total, 1LL));
    int *rv = (int *)raw.reserve(sizeof(int) * (size_t)std::max(total, 1LL));
    MFEM_CUDA(cudaMemcpyAsync(ptr, hIndex, sizeof(int) * ((size_t)N + 1), cudaMemcpyHostToDevice,
                              c.stream));
    int *st = status_ptr(c);
    MFEM_CUDA(cudaMemsetAsync(st, 0, sizeof(int), c.stream));
    if (total > 0) {
        MFEM_CUDA(cudaMemcpyAsync(rv, hValue, sizeof(int) * (size_t)total, cudaMemcpyHostToDevice,
                                  c.stream));
        k_caller_incidence<<<blocks_for(total, kThreads), kThreads, 0, c.stream>>>(rv, ne, total,
                                                                                 c.nbElem, st);
        check_launch("k_caller_incidence");
    }
    int bad = 0;
    read_status(c, &bad, 1);
    MFEM_REQUIRE(!(bad & kBadIndex), MFEM_ERR_INVALID_ARG,
                 "nodeToElem holds an element id outside [0, nbElem)");
    build_rows(c, MFEM_ORDER_REFERENCE, ptr, ne);
    // the caller's lists are freed on return: the row kernels must be done
    MFEM_CUDA(cudaStreamSynchronize(c.stream));
}

__global__ void k_diag_from_pattern(const int *__restrict__ rowPtr, const int *__restrict__ col,
                                    int nbNodes, int *diagPos) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nbNodes) return;
    int dp = -1;
    for (int p = rowPtr[r]; p < rowPtr[r + 1]; p++)
        if (col[p] == r) { dp = p; break; }
    diagPos[r] = dp;
}

__global__ void k_check_sorted(const int *__restrict__ rowPtr, const int *__restrict__ col,
                               int nbNodes, int *notSorted) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nbNodes) return;
    for (int p = rowPtr[r] + 1; p < rowPtr[r + 1]; p++)
        if (col[p] <= col[p - 1]) { atomicOr(notSorted, 1); return; }
}

void adopt_pattern(Context &c, const int *hRow, const int *hCol, int nnz) {
    const int N = c.nbNodes;
    MFEM_REQUIRE(hRow[0] == 0 && hRow[N] == nnz, MFEM_ERR_PATTERN,
                 "row pointers do not span nbEdges");
    for (int i = 0; i < N; i++)
        MFEM_REQUIRE(hRow[i + 1] >= hRow[i], MFEM_ERR_PATTERN, "row pointers decrease");
    build_incidence(c);
    int *rowPtr = (int *)c.rowPtr.reserve(sizeof(int) * (N + 1));
    int *col = (int *)c.col.reserve(sizeof(int) * (size_t)nnz);
    int *diag = (int *)c.diagPos.reserve(sizeof(int) * (size_t)N);
    int *st = status_ptr(c);
    MFEM_CUDA(cudaMemsetAsync(st, 0, sizeof(int) * 2, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(rowPtr, hRow, sizeof(int) * (N + 1), cudaMemcpyHostToDevice, c.stream));
    int *colIn = (int *)c.scratch.reserve(sizeof(int) * (size_t)nnz);
    MFEM_CUDA(cudaMemcpyAsync(colIn, hCol, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, c.stream));
    k_to_zero_based<<<blocks_for(nnz, kThreads), kThreads, 0, c.stream>>>(colIn, col, nnz, N, st);
    check_launch("k_to_zero_based");
    k_diag_from_pattern<<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(rowPtr, col, N, diag);
    check_launch("k_diag_from_pattern");
    k_check_sorted<<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(rowPtr, col, N, st + 1);
    check_launch("k_check_sorted");
    int h[2] = {0, 0};
    read_status(c, h, 2);
    MFEM_REQUIRE(!(h[0] & kBadIndex), MFEM_ERR_PATTERN, "column index out of range");
    c.nnz = nnz;
    c.order = h[1] ? MFEM_ORDER_REFERENCE : MFEM_ORDER_SORTED;   // unsorted: linear search
    c.hasPattern = true;
    c.hasElemPos = false;
    c.gather.built = false;
    c.tiles.built = false;
}

void build_elem_pos(Context &c) {
    MFEM_REQUIRE(c.hasPattern, MFEM_ERR_STATE, "no pattern");
    if (c.hasElemPos) return;
    const long long n4 = 4LL * c.nbElem;
    int *ep = (int *)c.elemPos.reserve(sizeof(int) * (size_t)n4 * 4);
    int *st = status_ptr(c);
    MFEM_CUDA(cudaMemsetAsync(st, 0, sizeof(int), c.stream));
    k_elem_pos<<<blocks_for(n4, kThreads), kThreads, 0, c.stream>>>(
        c.e2n.as<int>(), n4, c.rowPtr.as<int>(), c.col.as<int>(),
        c.order == MFEM_ORDER_SORTED, ep, st);
    check_launch("k_elem_pos");
    check_status(c, "create_elemToEdge");
    c.hasElemPos = true;
}

void build_gather_plan(Context &c) {
    MFEM_REQUIRE(c.hasPattern, MFEM_ERR_STATE, "no pattern");
    if (c.gather.built) return;
    build_incidence(c);
    const int N = c.nbNodes, nnz = c.nnz;
    const bool sorted = c.order == MFEM_ORDER_SORTED;
    GatherPlan &g = c.gather;
    int *st = status_ptr(c);
    MFEM_CUDA(cudaMemsetAsync(st, 0, sizeof(int), c.stream));
    // scratch layout: rowOf[nnz] | fill[max(nnz, N)] (then unit / node keys) |
    // tpos[nnz] | keyCount[nKeys + 1]
    const long long nKeys = ((long long)(c.nbElem >> kOwnerShift) + 1) * kDiagCountBins;
    MFEM_REQUIRE(nKeys < (1LL << 31), MFEM_ERR_CAPACITY, "gather plan: too many elements");
    const size_t nFill = std::max<size_t>((size_t)nnz, (size_t)N);
    int *work = (int *)c.scratch2.reserve(sizeof(int) * ((size_t)nnz * 2 + nFill + (size_t)nKeys + 1));
    int *rowOf = work, *fill = work + nnz, *tpos = fill + nFill;
    int *keyCount = tpos + nnz;
    int *start = (int *)g.unitStart.reserve(sizeof(int) * ((size_t)nnz + 1));
    int *tmp = (int *)c.scanTmp.reserve(sizeof(int) * scan_tmp_elems(std::max<long long>(nnz, nKeys) + 1));
    const int *ptr = c.nodeElemPtr.as<int>(), *ne = c.nodeElem.as<int>(), *e2n = c.e2n.as<int>();
    const int *rowPtr = c.rowPtr.as<int>(), *col = c.col.as<int>();

    k_plan_count<<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(ptr, ne, e2n, rowPtr, col, sorted, N, start, st);
    check_launch("k_plan_count");
    exclusive_scan_i32(start, start, nnz, tmp, c.stream);
    int total = 0;
    MFEM_CUDA(cudaMemcpyAsync(&total, start + nnz, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaStreamSynchronize(c.stream));
    check_status(c, "gather plan");
    MFEM_REQUIRE(total == 10LL * c.nbElem, MFEM_ERR_PATTERN, "gather plan: contribution count mismatch");
    unsigned *contrib = (unsigned *)g.contrib.reserve(sizeof(unsigned) * (size_t)total);
    k_plan_fill<<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(ptr, ne, e2n, rowPtr, col, sorted, N, start, fill, contrib, tpos, st);
    check_launch("k_plan_fill");
    k_row_of<<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(rowPtr, N, rowOf);
    check_launch("k_row_of");
    // off-diagonal units
    const int nKeysU = (int)(nKeys / kDiagCountBins * kUnitCountBins);
    int *key = fill;
    MFEM_CUDA(cudaMemsetAsync(keyCount, 0, sizeof(int) * ((size_t)nKeysU + 1), c.stream));
    k_unit_key<<<blocks_for(nnz, kThreads), kThreads, 0, c.stream>>>(rowOf, col, start, contrib, nnz, key, keyCount);
    check_launch("k_unit_key");
    exclusive_scan_i32(keyCount, keyCount, nKeysU, tmp, c.stream);
    int nEdge = 0;
    MFEM_CUDA(cudaMemcpyAsync(&nEdge, keyCount + nKeysU, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaStreamSynchronize(c.stream));
    int2 *upos = (int2 *)g.unitPos.reserve(sizeof(int2) * (size_t)(nEdge > 0 ? nEdge : 1));
    k_unit_place<<<blocks_for(nnz, kThreads), kThreads, 0, c.stream>>>(key, tpos, nnz, keyCount, upos);
    check_launch("k_unit_place");
    // diagonal units
    int *dnode = (int *)g.diagNode.reserve(sizeof(int) * (size_t)N);
    MFEM_CUDA(cudaMemsetAsync(keyCount, 0, sizeof(int) * ((size_t)nKeys + 1), c.stream));
    k_diag_key<<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(ptr, ne, N, key, keyCount);
    check_launch("k_diag_key");
    exclusive_scan_i32(keyCount, keyCount, nKeys, tmp, c.stream);
    k_diag_place<<<blocks_for(N, kThreads), kThreads, 0, c.stream>>>(key, N, keyCount, dnode);
    check_launch("k_diag_place");
    check_status(c, "gather plan");
    g.nUnits = nEdge;
    g.nContrib = total;
    g.nDiagUnits = N;
    g.built = true;
}

}  // namespace mfem
