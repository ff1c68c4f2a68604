// Element colouring on the device.
//
// Replaces coloring_creation (src/coloring.cc:84-109), whose greedy first-fit
// pass (create_longest_color_part, coloring.cc:46-81) is inherently sequential,
// by Jones-Plassmann: every element gets a hashed priority; in each round an
// uncoloured element whose priority beats all its uncoloured neighbours takes the
// smallest colour not used by its coloured neighbours (a 128-bit mask, the
// reference's MAX_COLOR = 128 limit, coloring.cc:22 and :66-69).  Neighbours are
// elements sharing a node (the reference's DC_create_elemToElem adjacency).
// Then a stable counting sort by colour gives the colour index
// (fill_color_index, coloring.cc:27-42) and the permutation to colour order
// (DC_create_permutation, called at coloring.cc:107).
#include <utility>

#include "context.h"

namespace mfem {

namespace {

constexpr int kThreads = 256;
constexpr int kTile = 2048;   // elements per warp in the stable placement

__device__ __forceinline__ unsigned prio(unsigned e, unsigned long long seed) {
    unsigned long long z = (unsigned long long)e + seed * 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return (unsigned)(z ^ (z >> 31));
}

// One Jones-Plassmann round.  Colours are read from the previous round's array
// and written to a new one, so the result does not depend on thread timing.
__global__ void k_jp_round(const int *__restrict__ e2n, const int *__restrict__ ptr,
                           const int *__restrict__ nodeElem, int nbElem,
                           unsigned long long seed, const int *__restrict__ cin,
                           int *__restrict__ cout, int *remaining, int *overflow) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nbElem) return;
    if (cin[e] >= 0) {
        cout[e] = cin[e];
        return;
    }
    const unsigned pe = prio(e, seed);
    unsigned used[4] = {0u, 0u, 0u, 0u};
    bool best = true;
    for (int k = 0; k < 4 && best; k++) {
        const int n = e2n[4 * e + k];
        for (int q = ptr[n]; q < ptr[n + 1]; q++) {
            const int f = nodeElem[q] >> 2;
            if (f == e) continue;
            const int cf = cin[f];
            if (cf >= 0) {
                used[cf >> 5] |= 1u << (cf & 31);
            } else {
                const unsigned pf = prio(f, seed);
                if (pf > pe || (pf == pe && f > e)) { best = false; break; }
            }
        }
    }
    if (!best) {
        cout[e] = -1;
        atomicAdd(remaining, 1);
        return;
    }
    int cidx = -1;
#pragma unroll
    for (int w = 0; w < 4; w++) {
        if (cidx < 0 && used[w] != 0xffffffffu) cidx = 32 * w + __ffs(~used[w]) - 1;
    }
    if (cidx < 0) {
        atomicOr(overflow, 1);
        cidx = 127;   // keeps the loop finite; the call reports MFEM_ERR_COLORS
    }
    cout[e] = cidx;
}

// One warp per tile: per-colour counts of the tile, stored colour-major.
__global__ void k_color_tile_hist(const int *__restrict__ color, int nbElem, int nTiles,
                                  int nColors, int *hist) {
    const int tile = blockIdx.x;
    const int lane = threadIdx.x;
    __shared__ int cnt[128];
    for (int c = lane; c < 128; c += 32) cnt[c] = 0;
    __syncwarp();
    const int b = tile * kTile, e = min(b + kTile, nbElem);
    for (int i = b + lane; i < e; i += 32) atomicAdd(&cnt[color[i]], 1);
    __syncwarp();
    for (int c = lane; c < nColors; c += 32) hist[(size_t)c * nTiles + tile] = cnt[c];
}

// Stable placement: element order is kept within every colour.
__global__ void k_color_tile_place(const int *__restrict__ color, int nbElem, int nTiles,
                                   const int *__restrict__ offs, int *colorElems,
                                   int *colorPerm) {
    const int tile = blockIdx.x;
    const int lane = threadIdx.x;
    __shared__ int run[128];
    for (int c = lane; c < 128; c += 32) run[c] = 0;
    __syncwarp();
    const int b = tile * kTile, e = min(b + kTile, nbElem);
    const unsigned lt = (1u << lane) - 1u;
    for (int base = b; base < e; base += 32) {
        const int i = base + lane;
        const bool ok = i < e;
        const int c = ok ? color[i] : -1;
        const unsigned m = __match_any_sync(0xffffffffu, c);
        const int rank = __popc(m & lt);
        int pos = 0;
        if (ok) pos = offs[(size_t)c * nTiles + tile] + run[c] + rank;
        __syncwarp();
        if (ok && rank == 0) run[c] += __popc(m);
        __syncwarp();
        if (ok) {
            colorElems[pos] = i;
            colorPerm[i] = pos;
        }
    }
}

}  // namespace

void build_coloring(Context &c, unsigned long long seed) {
    build_incidence(c);
    const int E = c.nbElem;
    Coloring &col = c.coloring;
    int *color = (int *)col.color.reserve(sizeof(int) * (size_t)E);
    int *other = (int *)c.scratch.reserve(sizeof(int) * (size_t)E);
    MFEM_CUDA(cudaMemsetAsync(color, 0xff, sizeof(int) * (size_t)E, c.stream));
    int *st = status_ptr(c);
    int rounds = 0;
    for (;;) {
        MFEM_CUDA(cudaMemsetAsync(st, 0, sizeof(int) * 2, c.stream));
        k_jp_round<<<blocks_for(E, kThreads), kThreads, 0, c.stream>>>(
            c.e2n.as<int>(), c.nodeElemPtr.as<int>(), c.nodeElem.as<int>(), E, seed, color,
            other, st, st + 1);
        check_launch("k_jp_round");
        std::swap(color, other);
        int h[2];
        read_status(c, h, 2);
        MFEM_REQUIRE(!h[1], MFEM_ERR_COLORS, "Not enough colors (more than 128 needed)");
        rounds++;
        if (h[0] == 0) break;
        MFEM_REQUIRE(rounds < 100000, MFEM_ERR_COLORS, "colouring did not converge");
    }
    if (color != col.color.as<int>())
        MFEM_CUDA(cudaMemcpyAsync(col.color.as<int>(), color, sizeof(int) * (size_t)E,
                                  cudaMemcpyDeviceToDevice, c.stream));
    color = col.color.as<int>();
    MFEM_CUDA(cudaStreamSynchronize(c.stream));   // `other` may be released below
    // number of colours = max colour + 1
    const int nTiles = (E + kTile - 1) / kTile;
    int *hist = (int *)c.scratch.reserve(sizeof(int) * ((size_t)128 * nTiles + 1));
    int *tmp = (int *)c.scanTmp.reserve(sizeof(int) * scan_tmp_elems((long long)128 * nTiles + 1));
    k_color_tile_hist<<<nTiles, 32, 0, c.stream>>>(color, E, nTiles, 128, hist);
    check_launch("k_color_tile_hist");
    std::vector<int> h((size_t)128 * nTiles);
    MFEM_CUDA(cudaMemcpyAsync(h.data(), hist, sizeof(int) * h.size(), cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaStreamSynchronize(c.stream));
    int nColors = 0;
    col.hOffsets.assign(129, 0);
    for (int k = 0; k < 128; k++) {
        long long s = 0;
        for (int t = 0; t < nTiles; t++) s += h[(size_t)k * nTiles + t];
        if (s > 0) nColors = k + 1;
        col.hOffsets[k + 1] = col.hOffsets[k] + (int)s;
    }
    col.hOffsets.resize(nColors + 1);
    exclusive_scan_i32(hist, hist, (long long)nColors * nTiles, tmp, c.stream);
    int *elems = (int *)col.colorElems.reserve(sizeof(int) * (size_t)E);
    int *perm = (int *)col.perm.reserve(sizeof(int) * (size_t)E);
    k_color_tile_place<<<nTiles, 32, 0, c.stream>>>(color, E, nTiles, hist, elems, perm);
    check_launch("k_color_tile_place");
    col.nbColors = nColors;
    col.built = true;
}

}  // namespace mfem
