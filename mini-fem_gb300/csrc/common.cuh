// Shared helpers of the sm_103a assembly library: status codes, device buffers,
// launch helpers and the exclusive scan used by the setup kernels.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <stdexcept>
#include <utility>

#include "mfem_gpu.h"

namespace mfem {

// Error carried from any internal layer up to the C entry points, which turn it
// into an MFEM_ERR_* code and keep the message for mfem_last_error().
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

#define MFEM_CUDA(call)                                                              \
    do {                                                                             \
        cudaError_t err_ = (call);                                                   \
        if (err_ != cudaSuccess)                                                     \
            throw ::mfem::Error(MFEM_ERR_CUDA, std::string(#call) + ": " +          \
                                cudaGetErrorString(err_));                          \
    } while (0)

#define MFEM_REQUIRE(cond, code, msg)                                                \
    do {                                                                             \
        if (!(cond)) throw ::mfem::Error((code), (msg));                             \
    } while (0)

// Grow-only device allocation owned by the context.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    void release() {
        if (ptr) cudaFree(ptr);
        ptr = nullptr;
        bytes = 0;
    }
    void *reserve(size_t n) {
        if (n == 0) n = 16;
        if (n > bytes) {
            release();
            MFEM_CUDA(cudaMalloc(&ptr, n));
            bytes = n;
        }
        return ptr;
    }
    template <class T> T *as() const { return static_cast<T *>(ptr); }
    void swap(DevBuf &o) {
        std::swap(ptr, o.ptr);
        std::swap(bytes, o.bytes);
    }
};

inline unsigned blocks_for(long long n, int threads) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 0x7fffffffLL) b = 0x7fffffffLL;
    return (unsigned)b;
}

inline void check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        throw Error(MFEM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Exclusive prefix sum of n int32 values: out[i] = sum(in[0..i)), out[n] = total.
// in and out may alias.  tmp must hold scan_tmp_elems(n) ints.  Returns nothing;
// the total is read back by the caller when needed.
size_t scan_tmp_elems(long long n);
void exclusive_scan_i32(const int *in, int *out, long long n, int *tmp, cudaStream_t s);

}  // namespace mfem
