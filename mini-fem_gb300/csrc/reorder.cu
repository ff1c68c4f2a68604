// Node renumbering: reverse Cuthill-McKee on the CSR pattern of the mesh.
//
// No counterpart in the reference, whose locality comes from its D&C tree
// permutations (DC-lib, src/main.cc:155-206).  RCM is one of the renumberings
// the tuner compares (identity vs RCM): it narrows the bandwidth of the matrix,
// so rows that are close in number share elements and cache lines.  Setup-time
// host code on the pattern already built on the device.
#include <algorithm>
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

}  // namespace mfem

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
