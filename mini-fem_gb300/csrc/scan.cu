// Exclusive prefix sum for the setup kernels (row pointers, incidence offsets,
// gather-plan offsets).  Three phases: per-tile sums, one-block scan of the tile
// sums, per-tile scan with the tile offset added.
#include "common.cuh"

namespace mfem {

namespace {

constexpr int kThreads = 512;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

__global__ void k_tile_sums(const int *__restrict__ in, long long n, int *__restrict__ sums) {
    long long base = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kItems;
    int s = 0;
#pragma unroll
    for (int i = 0; i < kItems; i++)
        if (base + i < n) s += in[base + i];
    __shared__ int red[kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        int t = (threadIdx.x < kThreads / 32) ? red[threadIdx.x] : 0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) sums[blockIdx.x] = t;
    }
}

// Single block, in place: data[i] = sum(data[0..i)), data[n] = total.
__global__ void k_scan_one_block(int *data, int n) {
    __shared__ int carry;
    __shared__ int warpSums[kThreads / 32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int base = 0; base < n; base += kThreads) {
        int i = base + threadIdx.x;
        int v = (i < n) ? data[i] : 0;
        int incl = warp_incl_scan(v);
        if (lane == 31) warpSums[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            int w = (lane < kThreads / 32) ? warpSums[lane] : 0;
            int wi = warp_incl_scan(w);
            if (lane < kThreads / 32) warpSums[lane] = wi - w;
        }
        __syncthreads();
        int excl = incl - v + warpSums[warp] + carry;
        if (i < n) data[i] = excl;
        __syncthreads();
        if (threadIdx.x == kThreads - 1) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) data[n] = carry;
}

__global__ void k_tile_scan(const int *in, int *out, long long n,
                            const int *__restrict__ tileOffsets) {
    __shared__ int warpSums[kThreads / 32];
    long long base = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kItems;
    int v[kItems];
    int s = 0;
#pragma unroll
    for (int i = 0; i < kItems; i++) {
        v[i] = (base + i < n) ? in[base + i] : 0;
        s += v[i];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int incl = warp_incl_scan(s);
    if (lane == 31) warpSums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = (lane < kThreads / 32) ? warpSums[lane] : 0;
        int wi = warp_incl_scan(w);
        if (lane < kThreads / 32) warpSums[lane] = wi - w;
    }
    __syncthreads();
    int run = incl - s + warpSums[warp] + tileOffsets[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kItems; i++) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
    if (base < n && base + kItems >= n) out[n] = run;   // thread holding the last item
}

}  // namespace

size_t scan_tmp_elems(long long n) {
    long long tiles = (n + kTile - 1) / kTile;
    return (size_t)(tiles + 1);
}

void exclusive_scan_i32(const int *in, int *out, long long n, int *tmp, cudaStream_t s) {
    if (n <= 0) {
        MFEM_CUDA(cudaMemsetAsync(out, 0, sizeof(int), s));
        return;
    }
    long long tiles = (n + kTile - 1) / kTile;
    MFEM_REQUIRE(tiles < (1LL << 31), MFEM_ERR_CAPACITY, "scan too large");
    k_tile_sums<<<(unsigned)tiles, kThreads, 0, s>>>(in, n, tmp);
    check_launch("k_tile_sums");
    k_scan_one_block<<<1, kThreads, 0, s>>>(tmp, (int)tiles);
    check_launch("k_scan_one_block");
    k_tile_scan<<<(unsigned)tiles, kThreads, 0, s>>>(in, out, n, tmp);
    check_launch("k_tile_scan");
}

}  // namespace mfem
