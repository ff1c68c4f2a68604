// Node renumbering: reverse Cuthill-McKee on the CSR pattern of the mesh.
//
// No counterpart in the reference, whose locality comes from its D&C tree
// permutations (DC-lib, src/main.cc:155-206).  RCM is one of the renumberings
// the tuner compares (identity vs RCM): it narrows the bandwidth of the matrix,
// so rows that are close in number share elements and cache lines.  Setup-time
// host code on the pattern already built on the device.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "context.h"

namespace mfem {

namespace {

// Breadth-first levels from `root`; returns the last level and fills `level`.
int bfs_levels(const std::vector<int> &ptr, const std::vector<int> &adj, int root,
               std::vector<int> &level, std::vector<int> &lastLevel) {
    std::fill(level.begin(), level.end(), -1);
    std::vector<int> frontier{root}, next;
    level[root] = 0;
    int depth = 0;
    lastLevel = frontier;
    while (!frontier.empty()) {
        next.clear();
        for (int u : frontier)
            for (int q = ptr[u]; q < ptr[u + 1]; q++) {
                const int v = adj[q];
                if (level[v] < 0) {
                    level[v] = depth + 1;
                    next.push_back(v);
                }
            }
        if (next.empty()) break;
        depth++;
        lastLevel = next;
        std::swap(frontier, next);
    }
    return depth;
}

}  // namespace

void rcm_permutation(Context &c, int *newOfOld) {
    MFEM_REQUIRE(c.hasPattern, MFEM_ERR_STATE, "no CSR pattern");
    const int N = c.nbNodes, nnz = c.nnz;
    std::vector<int> ptr(N + 1), col((size_t)nnz);
    MFEM_CUDA(cudaMemcpyAsync(ptr.data(), c.rowPtr.ptr, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaMemcpyAsync(col.data(), c.col.ptr, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaStreamSynchronize(c.stream));
    // adjacency without the diagonal
    std::vector<int> aptr(N + 1, 0), adj;
    adj.reserve((size_t)nnz);
    for (int i = 0; i < N; i++) {
        for (int q = ptr[i]; q < ptr[i + 1]; q++)
            if (col[q] != i) adj.push_back(col[q]);
        aptr[i + 1] = (int)adj.size();
    }
    std::vector<int> deg(N);
    for (int i = 0; i < N; i++) deg[i] = aptr[i + 1] - aptr[i];

    std::vector<char> placed(N, 0);
    std::vector<int> order;
    order.reserve(N);
    std::vector<int> level(N), last, nb;
    int searchFrom = 0;
    while ((int)order.size() < N) {
        // unplaced node of smallest degree starts the next component
        int root = -1;
        for (int i = searchFrom; i < N; i++)
            if (!placed[i] && (root < 0 || deg[i] < deg[root])) root = i;
        // pseudo-peripheral node (George-Liu): walk to a far node of least degree
        int ecc = bfs_levels(aptr, adj, root, level, last);
        for (int it = 0; it < 8; it++) {
            int cand = last[0];
            for (int v : last)
                if (deg[v] < deg[cand]) cand = v;
            std::vector<int> l2;
            const int e2 = bfs_levels(aptr, adj, cand, level, l2);
            if (e2 <= ecc) break;
            ecc = e2;
            root = cand;
            last = l2;
        }
        // Cuthill-McKee from root
        size_t head = order.size();
        order.push_back(root);
        placed[root] = 1;
        while (head < order.size()) {
            const int u = order[head++];
            nb.clear();
            for (int q = aptr[u]; q < aptr[u + 1]; q++)
                if (!placed[adj[q]]) {
                    placed[adj[q]] = 1;
                    nb.push_back(adj[q]);
                }
            std::sort(nb.begin(), nb.end(), [&](int x, int y) {
                return deg[x] != deg[y] ? deg[x] < deg[y] : x < y;
            });
            order.insert(order.end(), nb.begin(), nb.end());
        }
        while (searchFrom < N && placed[searchFrom]) searchFrom++;
    }
    // reverse
    for (int k = 0; k < N; k++) newOfOld[order[N - 1 - k]] = k;
}

// Locality orderings of the nodes from their coordinates (no graph needed):
// Morton (Z-order) of the coordinates quantised to 21 bits per axis, or
// recursive coordinate bisection -- split the node set at the median of its
// longest bounding-box axis, recursively, and number the leaves (at most
// kLeaf nodes, Morton order inside) depth first.  The bisection tree plays the
// part of the reference's D&C tree ordering (src/main.cc:155-206, DC-lib,
// absent), derived from the geometry instead of the element graph.
namespace {

constexpr int kLeaf = 64;

uint64_t spread21(uint64_t v) {   // 21 bits -> every third bit of 63
    v &= 0x1fffff;
    v = (v | v << 32) & 0x1f00000000ffffULL;
    v = (v | v << 16) & 0x1f0000ff0000ffULL;
    v = (v | v << 8) & 0x100f00f00f00f00fULL;
    v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
    v = (v | v << 2) & 0x1249249249249249ULL;
    return v;
}

std::vector<uint64_t> morton_keys(const std::vector<double> &xyz, int N) {
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int i = 0; i < N; i++)
        for (int d = 0; d < 3; d++) {
            lo[d] = std::min(lo[d], xyz[3 * (size_t)i + d]);
            hi[d] = std::max(hi[d], xyz[3 * (size_t)i + d]);
        }
    std::vector<uint64_t> key(N);
    for (int i = 0; i < N; i++) {
        uint64_t k = 0;
        for (int d = 0; d < 3; d++) {
            const double span = hi[d] > lo[d] ? hi[d] - lo[d] : 1.0;
            const double f = (xyz[3 * (size_t)i + d] - lo[d]) / span;
            const uint64_t q = (uint64_t)std::min(2097151.0, std::max(0.0, f * 2097151.0));
            k |= spread21(q) << d;
        }
        key[i] = k;
    }
    return key;
}

void bisect(const std::vector<double> &xyz, const std::vector<uint64_t> &key, std::vector<int> &idx,
            size_t lo, size_t hi, std::vector<int> &order) {
    if (hi - lo <= (size_t)kLeaf) {
        std::sort(idx.begin() + lo, idx.begin() + hi, [&](int a, int b) {
            return key[a] != key[b] ? key[a] < key[b] : a < b;
        });
        order.insert(order.end(), idx.begin() + lo, idx.begin() + hi);
        return;
    }
    double bl[3] = {1e300, 1e300, 1e300}, bh[3] = {-1e300, -1e300, -1e300};
    for (size_t q = lo; q < hi; q++)
        for (int d = 0; d < 3; d++) {
            bl[d] = std::min(bl[d], xyz[3 * (size_t)idx[q] + d]);
            bh[d] = std::max(bh[d], xyz[3 * (size_t)idx[q] + d]);
        }
    int ax = 0;
    for (int d = 1; d < 3; d++)
        if (bh[d] - bl[d] > bh[ax] - bl[ax]) ax = d;
    const size_t mid = lo + (hi - lo) / 2;
    std::nth_element(idx.begin() + lo, idx.begin() + mid, idx.begin() + hi, [&](int a, int b) {
        const double xa = xyz[3 * (size_t)a + ax], xb = xyz[3 * (size_t)b + ax];
        return xa != xb ? xa < xb : a < b;
    });
    bisect(xyz, key, idx, lo, mid, order);
    bisect(xyz, key, idx, mid, hi, order);
}

}  // namespace

void locality_permutation(Context &c, int kind, int *newOfOld) {
    MFEM_REQUIRE(c.hasCoords, MFEM_ERR_STATE, "no coordinates");
    MFEM_REQUIRE(kind == MFEM_LOCALITY_MORTON || kind == MFEM_LOCALITY_BISECTION, MFEM_ERR_INVALID_ARG,
                 "unknown locality ordering");
    const int N = c.nbNodes;
    std::vector<double> xyz((size_t)N * 3);
    MFEM_CUDA(cudaMemcpyAsync(xyz.data(), c.coord.ptr, xyz.size() * 8, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaStreamSynchronize(c.stream));
    const std::vector<uint64_t> key = morton_keys(xyz, N);
    std::vector<int> idx(N), order;
    for (int i = 0; i < N; i++) idx[i] = i;
    if (kind == MFEM_LOCALITY_MORTON) {
        std::sort(idx.begin(), idx.end(), [&](int a, int b) {
            return key[a] != key[b] ? key[a] < key[b] : a < b;
        });
        order.swap(idx);
    } else {
        order.reserve(N);
        bisect(xyz, key, idx, 0, (size_t)N, order);
    }
    for (int k = 0; k < N; k++) newOfOld[order[k]] = k;
}

}  // namespace mfem

extern "C" int mfem_locality_permutation(mfem_context *ctx, int kind, int *newOfOld) {
    if (!ctx || !newOfOld) return MFEM_ERR_INVALID_ARG;
    try {
        MFEM_CUDA(cudaSetDevice(ctx->c.device));
        mfem::locality_permutation(ctx->c, kind, newOfOld);
        ctx->c.lastError.clear();
        return MFEM_OK;
    } catch (const mfem::Error &e) {
        ctx->c.lastError = e.what();
        return e.code;
    }
}

extern "C" int mfem_rcm_permutation(mfem_context *ctx, int *newOfOld) {
    if (!ctx || !newOfOld) return MFEM_ERR_INVALID_ARG;
    try {
        MFEM_CUDA(cudaSetDevice(ctx->c.device));
        mfem::rcm_permutation(ctx->c, newOfOld);
        ctx->c.lastError.clear();
        return MFEM_OK;
    } catch (const mfem::Error &e) {
        ctx->c.lastError = e.what();
        return e.code;
    }
}
