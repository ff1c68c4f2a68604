// C entry points (include/mfem_gpu.h): argument checks, host<->device copies,
// and dispatch to the kernels.  Every entry point catches internal errors and
// returns a status; the message is kept for mfem_last_error().
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "context.h"

namespace mfem {

int *status_ptr(Context &c) { return c.status.as<int>(); }

void KernelTimer::begin(const char *name, cudaStream_t s) {
    if (!on) return;
    if (used == recs.size()) {
        Rec r{name, nullptr, nullptr};
        MFEM_CUDA(cudaEventCreate(&r.a));
        MFEM_CUDA(cudaEventCreate(&r.b));
        recs.push_back(r);
    }
    recs[used].name = name;
    MFEM_CUDA(cudaEventRecord(recs[used].a, s));
}

void KernelTimer::end(cudaStream_t s) {
    if (!on) return;
    MFEM_CUDA(cudaEventRecord(recs[used].b, s));
    used++;
}

KernelTimer::~KernelTimer() {
    for (auto &r : recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
}

void read_status(Context &c, int *h, int n) {
    MFEM_CUDA(cudaMemcpyAsync(h, c.status.as<int>(), sizeof(int) * n, cudaMemcpyDeviceToHost,
                              c.stream));
    MFEM_CUDA(cudaStreamSynchronize(c.stream));
}

void assemble_fp32(Context &c, int op, int strategy, bool fusePrec);

namespace {

__global__ void k_e2n_zero_based(const int *__restrict__ in, int *__restrict__ out,
                                 long long n, int nbNodes, int *bad) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int v = in[i] - 1;
    if (v < 0 || v >= nbNodes) {
        atomicOr(bad, 1);
        v = 0;
    }
    out[i] = v;
}

__global__ void k_plus_one(const int *__restrict__ in, int *__restrict__ out, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i] + 1;
}

// MARKF(nbNodes, 3), column-major (src/Fortran/e_cgmelissa.F:27-29) -> bit k of
// one byte per node.
__global__ void k_pack_mask(const int *__restrict__ cb, int nbNodes, unsigned char *mask) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbNodes) return;
    mask[i] = (unsigned char)((cb[i] != 0) | ((cb[i + (size_t)nbNodes] != 0) << 1) |
                              ((cb[i + 2 * (size_t)nbNodes] != 0) << 2));
}

__global__ void k_f32_to_f64(const float *__restrict__ in, double *__restrict__ out, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

int op_dim(int op) { return op == MFEM_OP_LAP ? 1 : 9; }

void require_mesh(Context &c) {
    MFEM_REQUIRE(c.nbElem > 0 && c.nbNodes > 0, MFEM_ERR_STATE, "no mesh set");
}

void require_pattern(Context &c) {
    require_mesh(c);
    MFEM_REQUIRE(c.hasPattern, MFEM_ERR_STATE, "no CSR pattern (create_nodeToNode first)");
}

// Order-dependent 64-bit fingerprint of n int32 values (four independent
// multiply-xorshift chains over 8-byte words, then folded): any change of the
// contents, a permutation of the element rows included, changes it with
// overwhelming probability.  Cost at 5.8M elements: a few ms on one core,
// against the 1 GB copy-out of the values that the same call makes.
unsigned long long fingerprint_i32(const int *a, long long n) {
    const unsigned long long K = 0x9E3779B97F4A7C15ULL;
    unsigned long long h[4] = {0x243F6A8885A308D3ULL, 0x13198A2E03707344ULL,
                               0xA4093822299F31D0ULL, 0x082EFA98EC4E6C89ULL};
    long long i = 0;
    for (; i + 8 <= n; i += 8)
        for (int l = 0; l < 4; l++) {
            unsigned long long w;
            std::memcpy(&w, a + i + 2 * l, sizeof(w));
            h[l] = (h[l] ^ w) * K;
            h[l] ^= h[l] >> 29;
        }
    for (; i < n; i++) {
        h[0] = (h[0] ^ (unsigned)a[i]) * K;
        h[0] ^= h[0] >> 29;
    }
    unsigned long long r = (unsigned long long)n;
    for (int l = 0; l < 4; l++) {
        r = (r ^ h[l]) * K;
        r ^= r >> 31;
    }
    return r;
}

void set_mesh(Context &c, const double *coord, const int *e2n, int nbElem, int nbNodes) {
    MFEM_REQUIRE(e2n, MFEM_ERR_INVALID_ARG, "null elemToNode");
    MFEM_REQUIRE(nbElem > 0 && nbNodes > 0, MFEM_ERR_INVALID_ARG, "empty mesh");
    MFEM_REQUIRE((long long)nbElem * 10 < (1LL << 31) && nbElem < (1 << 27),
                 MFEM_ERR_CAPACITY, "mesh too large for 32-bit plan indices");
    c.nbElem = nbElem;
    c.nbNodes = nbNodes;
    c.hasPattern = c.hasIncidence = c.hasElemPos = false;
    c.gather.built = false;
    c.tiles.built = false;
    c.coloring.built = false;
    c.halo.built = false;
    c.precBlocks = false;
    c.coefOp = -1;
    c.lameValid = false;
    c.hasMask = false;
    c.lastOp = -1;
    c.hostRow = c.hostCol = nullptr;
    double *dc = (double *)c.coord.reserve(sizeof(double) * 3 * (size_t)nbNodes);
    c.hasCoords = coord != nullptr;   // topology-only meshes get coordinates later
    if (coord)
        MFEM_CUDA(cudaMemcpyAsync(dc, coord, sizeof(double) * 3 * (size_t)nbNodes,
                                  cudaMemcpyHostToDevice, c.stream));
    const long long n4 = 4LL * nbElem;
    int *raw = (int *)c.scratch.reserve(sizeof(int) * (size_t)n4);
    int *de = (int *)c.e2n.reserve(sizeof(int) * (size_t)n4);
    MFEM_CUDA(cudaMemcpyAsync(raw, e2n, sizeof(int) * (size_t)n4, cudaMemcpyHostToDevice, c.stream));
    int *st = status_ptr(c);
    MFEM_CUDA(cudaMemsetAsync(st, 0, sizeof(int), c.stream));
    k_e2n_zero_based<<<blocks_for(n4, 256), 256, 0, c.stream>>>(raw, de, n4, nbNodes, st);
    check_launch("k_e2n_zero_based");
    int bad = 0;
    read_status(c, &bad, 1);
    if (bad) {
        c.nbElem = c.nbNodes = 0;
        throw Error(MFEM_ERR_INVALID_ARG, "elemToNode holds a node outside [1, nbNodes]");
    }
    c.hostE2n = e2n;
    c.hostE2nSig = fingerprint_i32(e2n, n4);
}

// Errors kernels report through the status words after they were enqueued:
// status[6] = a bounded wait gave up.
void check_async(Context &c) {
    int h[8];
    read_status(c, h, 8);
    if (h[6]) {
        MFEM_CUDA(cudaMemsetAsync(status_ptr(c) + 6, 0, sizeof(int), c.stream));
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
        throw Error(MFEM_ERR_TIMEOUT, "a device wait gave up (staged copies did not arrive in time); "
                                      "the results of that call are incomplete");
    }
}

void upload_coords(Context &c, const double *coord) {
    MFEM_REQUIRE(coord, MFEM_ERR_INVALID_ARG, "null coord");
    MFEM_CUDA(cudaMemcpyAsync(c.coord.as<double>(), coord, sizeof(double) * 3 * (size_t)c.nbNodes,
                              cudaMemcpyHostToDevice, c.stream));
    c.hasCoords = true;
}

void upload_coefficients(Context &c, int op, const double *coef) {
    require_mesh(c);
    MFEM_REQUIRE(op == MFEM_OP_LAP || op == MFEM_OP_ELA, MFEM_ERR_INVALID_ARG, "operatorID must be 0 or 1");
    c.lameValid = false;
    if (!coef) {
        c.coefOp = -1;
        return;
    }
    const size_t n = (size_t)c.nbElem * (op == MFEM_OP_LAP ? 1 : 2);
    double *d = (double *)c.coef.reserve(sizeof(double) * n);
    MFEM_CUDA(cudaMemcpyAsync(d, coef, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
    c.coefOp = op;
}

void download_col(Context &c, int *col) {
    int *tmp = (int *)c.scratch.reserve(sizeof(int) * (size_t)c.nnz);
    k_plus_one<<<blocks_for(c.nnz, 256), 256, 0, c.stream>>>(c.col.as<int>(), tmp, c.nnz);
    check_launch("k_plus_one");
    MFEM_CUDA(cudaMemcpyAsync(col, tmp, sizeof(int) * (size_t)c.nnz, cudaMemcpyDeviceToHost, c.stream));
}

void assemble(Context &c, int op, int precision, int strategy, bool fusePrec) {
    pipeline_guard(c);
    require_pattern(c);
    MFEM_REQUIRE(c.hasCoords, MFEM_ERR_STATE, "no coordinates (mfem_update_coords first)");
    MFEM_REQUIRE(op == MFEM_OP_LAP || op == MFEM_OP_ELA, MFEM_ERR_INVALID_ARG, "operatorID must be 0 or 1");
    MFEM_REQUIRE(precision == MFEM_FP64 || precision == MFEM_FP32, MFEM_ERR_INVALID_ARG, "unknown precision");
    if (strategy == MFEM_AUTO) strategy = MFEM_GATHER;
    MFEM_REQUIRE(strategy >= MFEM_GATHER && strategy <= MFEM_ATOMIC, MFEM_ERR_INVALID_ARG, "unknown strategy");
    c.precBlocks = false;
    if (precision == MFEM_FP64) assemble_fp64(c, op, strategy, fusePrec);
    else assemble_fp32(c, op, strategy, fusePrec);
    if (fusePrec && !c.precIsInit) {
        prec_init_fp64(c, op);
        prec_invert(c, op);
        c.precIsInit = true;
    }
}

template <class F>
int guarded(mfem_context *ctx, F &&f) {
    if (!ctx) return MFEM_ERR_INVALID_ARG;
    try {
        MFEM_CUDA(cudaSetDevice(ctx->c.device));
        f(ctx->c);
        ctx->c.lastError.clear();
        return MFEM_OK;
    } catch (const Error &e) {
        ctx->c.lastError = e.what();
        return e.code;
    } catch (const std::bad_alloc &) {
        ctx->c.lastError = "host allocation failed";
        return MFEM_ERR_CAPACITY;
    }
}

}  // namespace

Pipeline::~Pipeline() {
    if (copy) cudaStreamSynchronize(copy);
    for (auto &e : copied)
        if (e) cudaEventDestroy(e);
    if (computed) cudaEventDestroy(computed);
    if (copy) cudaStreamDestroy(copy);
    if (hostStatus) cudaFreeHost(hostStatus);
}

// Anything that writes the current result slot first waits (on the device) for
// the slot's pending copy-out.
void pipeline_guard(Context &c) {
    if (c.pipe && c.pipe->recorded[c.pipe->cur])
        MFEM_CUDA(cudaStreamWaitEvent(c.stream, c.pipe->copied[c.pipe->cur], 0));
}

namespace {

Pipeline &pipeline(Context &c) {
    if (!c.pipe) {
        auto p = std::make_unique<Pipeline>();
        MFEM_CUDA(cudaStreamCreateWithFlags(&p->copy, cudaStreamNonBlocking));
        MFEM_CUDA(cudaEventCreateWithFlags(&p->computed, cudaEventDisableTiming));
        for (auto &e : p->copied) MFEM_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        MFEM_CUDA(cudaMallocHost(&p->hostStatus, sizeof(int) * 16));
        for (int i = 0; i < 16; i++) p->hostStatus[i] = 0;
        c.pipe = std::move(p);
    }
    return *c.pipe;
}

// One pipelined step (mfem_step_async).
long long step_async(Context &c, int op, int precision, int strategy, const double *coord,
                     const double *coef, void *hostValues, double *hostPrec) {
    require_pattern(c);
    MFEM_REQUIRE(hostValues, MFEM_ERR_INVALID_ARG, "null host values");
    Pipeline &P = pipeline(c);
    const long long t = P.next;
    if (t > 0) {
        // the other slot becomes current; the previous step's results stay in
        // the spare slot while they are copied out
        c.values.swap(P.spareValues);
        c.prec.swap(P.sparePrec);
        P.cur ^= 1;
    }
    // a slot that must grow (first use of a precision with larger values) is
    // reallocated on the host: its last copy-out has to be finished first
    const size_t needValues = (size_t)c.nnz * op_dim(op) * (precision == MFEM_FP32 ? 4 : 8);
    const size_t needPrec = sizeof(double) * (size_t)c.nbNodes * op_dim(op);
    if (P.recorded[P.cur] && (c.values.bytes < needValues || c.prec.bytes < needPrec))
        MFEM_CUDA(cudaEventSynchronize(P.copied[P.cur]));
    if (coord) upload_coords(c, coord);
    if (coef) upload_coefficients(c, op, coef);
    assemble(c, op, precision, strategy, hostPrec != nullptr);   // waits for the slot's last copy-out
    int *hs = P.hostStatus + 8 * P.cur;
    MFEM_CUDA(cudaMemcpyAsync(hs, status_ptr(c), sizeof(int) * 8, cudaMemcpyDeviceToHost, c.stream));
    MFEM_CUDA(cudaEventRecord(P.computed, c.stream));
    MFEM_CUDA(cudaStreamWaitEvent(P.copy, P.computed, 0));
    const size_t n = (size_t)c.nnz * op_dim(op);
    MFEM_CUDA(cudaMemcpyAsync(hostValues, c.values.ptr, n * (precision == MFEM_FP32 ? 4 : 8),
                              cudaMemcpyDeviceToHost, P.copy));
    if (hostPrec)
        MFEM_CUDA(cudaMemcpyAsync(hostPrec, c.prec.ptr, sizeof(double) * (size_t)c.nbNodes * op_dim(op),
                                  cudaMemcpyDeviceToHost, P.copy));
    MFEM_CUDA(cudaEventRecord(P.copied[P.cur], P.copy));
    P.recorded[P.cur] = true;
    P.next = t + 1;
    return t;
}

void wait_step(Context &c, long long ticket) {
    MFEM_REQUIRE(c.pipe && ticket >= 0 && ticket < c.pipe->next, MFEM_ERR_INVALID_ARG, "unknown ticket");
    Pipeline &P = *c.pipe;
    // the slot's event was recorded by this step or by a later one (stream order)
    const int slot = (P.cur + (int)((P.next - 1 - ticket) & 1)) & 1;
    MFEM_CUDA(cudaEventSynchronize(P.copied[slot]));
    const int *hs = P.hostStatus + 8 * slot;
    if (hs[6]) {
        MFEM_CUDA(cudaMemsetAsync(status_ptr(c) + 6, 0, sizeof(int), c.stream));
        throw Error(MFEM_ERR_TIMEOUT, "a device wait gave up (staged copies did not arrive in time); "
                                      "the results of that step are incomplete");
    }
}

}  // namespace
}  // namespace mfem

using mfem::Context;
using mfem::Error;

extern "C" {

int mfem_abi_version(void) { return MFEM_ABI_VERSION; }

const char *mfem_status_string(int s) {
    switch (s) {
    case MFEM_OK: return "ok";
    case MFEM_ERR_INVALID_ARG: return "invalid argument";
    case MFEM_ERR_CUDA: return "CUDA error";
    case MFEM_ERR_NO_DEVICE: return "no CUDA device";
    case MFEM_ERR_STATE: return "call out of order";
    case MFEM_ERR_PATTERN: return "CSR pattern mismatch";
    case MFEM_ERR_COLORS: return "Not enough colors";
    case MFEM_ERR_CAPACITY: return "capacity exceeded";
    case MFEM_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
    }
}

const char *mfem_last_error(const mfem_context *ctx) {
    return ctx ? ctx->c.lastError.c_str() : "null context";
}

int mfem_create(mfem_context **out, int device) {
    if (!out) return MFEM_ERR_INVALID_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        cudaGetLastError();
        return MFEM_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= n) return MFEM_ERR_INVALID_ARG;
    mfem_context *ctx = new (std::nothrow) mfem_context;
    if (!ctx) return MFEM_ERR_CAPACITY;
    ctx->c.device = device;
    int rc = mfem::guarded(ctx, [](Context &c) {
        MFEM_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        c.status.reserve(sizeof(int) * 8);
        MFEM_CUDA(cudaMemsetAsync(c.status.ptr, 0, sizeof(int) * 8, c.stream));
    });
    if (rc != MFEM_OK) {
        delete ctx;
        return rc;
    }
    *out = ctx;
    return MFEM_OK;
}

int mfem_destroy(mfem_context *ctx) {
    if (!ctx) return MFEM_ERR_INVALID_ARG;
    cudaSetDevice(ctx->c.device);
    if (ctx->c.side) {
        cudaStreamSynchronize(ctx->c.side);
        cudaStreamDestroy(ctx->c.side);
    }
    if (ctx->c.sideFork) cudaEventDestroy(ctx->c.sideFork);
    if (ctx->c.sideJoin) cudaEventDestroy(ctx->c.sideJoin);
    if (ctx->c.stream) {
        cudaStreamSynchronize(ctx->c.stream);
        cudaStreamDestroy(ctx->c.stream);
    }
    delete ctx;
    return MFEM_OK;
}

int mfem_get_stream(mfem_context *ctx, void **stream) {
    if (!ctx || !stream) return MFEM_ERR_INVALID_ARG;
    *stream = (void *)ctx->c.stream;
    return MFEM_OK;
}

int mfem_set_mesh(mfem_context *ctx, const double *coord, const int *elemToNode, int nbElem,
                  int nbNodes) {
    return mfem::guarded(ctx, [&](Context &c) { mfem::set_mesh(c, coord, elemToNode, nbElem, nbNodes); });
}

int mfem_update_coords(mfem_context *ctx, const double *coord) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::require_mesh(c);
        mfem::upload_coords(c, coord);
    });
}

int mfem_create_nodeToNode(mfem_context *ctx, int order, int *row, int *col, int capacity,
                           int *nbEdges) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::require_mesh(c);
        mfem::build_pattern(c, order);
        if (nbEdges) *nbEdges = c.nnz;
        if (row)
            MFEM_CUDA(cudaMemcpyAsync(row, c.rowPtr.as<int>(), sizeof(int) * (c.nbNodes + 1),
                                      cudaMemcpyDeviceToHost, c.stream));
        if (col) {
            MFEM_REQUIRE(capacity >= c.nnz, MFEM_ERR_CAPACITY, "column buffer smaller than nnz");
            mfem::download_col(c, col);
        }
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
        c.hostRow = row;
        c.hostCol = col;
    });
}

int mfem_create_nodeToNode_incidence(mfem_context *ctx, const int *nodeToElemIndex,
                                     const int *nodeToElemValue, int *row, int *col,
                                     int capacity, int *nbEdges) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::require_mesh(c);
        mfem::build_pattern_from_incidence(c, nodeToElemIndex, nodeToElemValue);
        if (nbEdges) *nbEdges = c.nnz;
        if (row)
            MFEM_CUDA(cudaMemcpyAsync(row, c.rowPtr.as<int>(), sizeof(int) * (c.nbNodes + 1),
                                      cudaMemcpyDeviceToHost, c.stream));
        if (col) {
            MFEM_REQUIRE(capacity >= c.nnz, MFEM_ERR_CAPACITY, "column buffer smaller than nnz");
            mfem::download_col(c, col);
        }
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
        c.hostRow = row;
        c.hostCol = col;
    });
}

int mfem_create_elemToEdge(mfem_context *ctx, int *elemToEdge) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::require_pattern(c);
        MFEM_REQUIRE(elemToEdge, MFEM_ERR_INVALID_ARG, "null elemToEdge");
        mfem::build_elem_pos(c);
        MFEM_CUDA(cudaMemcpyAsync(elemToEdge, c.elemPos.as<int>(), sizeof(int) * 16 * (size_t)c.nbElem,
                                  cudaMemcpyDeviceToHost, c.stream));
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int mfem_set_pattern(mfem_context *ctx, const int *row, const int *col, int nbEdges) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::require_mesh(c);
        MFEM_REQUIRE(row && col && nbEdges > 0, MFEM_ERR_INVALID_ARG, "bad pattern arguments");
        mfem::adopt_pattern(c, row, col, nbEdges);
        // validates that every element pair is present
        mfem::build_elem_pos(c);
        c.hostRow = row;
        c.hostCol = col;
    });
}

int mfem_coloring_creation(mfem_context *ctx, unsigned long long seed, int *colorPerm,
                           int *colorIndex, int capacity, int *nbColors) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::require_mesh(c);
        mfem::build_coloring(c, seed);
        const int nc = c.coloring.nbColors;
        if (nbColors) *nbColors = nc;
        if (colorPerm)
            MFEM_CUDA(cudaMemcpyAsync(colorPerm, c.coloring.perm.as<int>(), sizeof(int) * (size_t)c.nbElem,
                                      cudaMemcpyDeviceToHost, c.stream));
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
        if (colorIndex) {
            MFEM_REQUIRE(capacity >= nc + 1, MFEM_ERR_CAPACITY, "colorIndex buffer too small");
            std::memcpy(colorIndex, c.coloring.hOffsets.data(), sizeof(int) * (nc + 1));
        }
    });
}

int mfem_set_coefficients(mfem_context *ctx, int operatorID, const double *coef) {
    return mfem::guarded(ctx, [&](Context &c) { mfem::upload_coefficients(c, operatorID, coef); });
}

int mfem_assemble(mfem_context *ctx, int operatorID, int precision, int strategy) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::assemble(c, operatorID, precision, strategy, false);
    });
}

int mfem_assemble_prec(mfem_context *ctx, int operatorID, int precision, int strategy) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::assemble(c, operatorID, precision, strategy, true);
    });
}

int mfem_set_check_bounds(mfem_context *ctx, const int *checkBounds) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::require_mesh(c);
        if (!checkBounds) {
            c.hasMask = false;
            return;
        }
        const int N = c.nbNodes;
        int *raw = (int *)c.scratch.reserve(sizeof(int) * 3 * (size_t)N);
        MFEM_CUDA(cudaMemcpyAsync(raw, checkBounds, sizeof(int) * 3 * (size_t)N,
                                  cudaMemcpyHostToDevice, c.stream));
        unsigned char *d = (unsigned char *)c.mask.reserve((size_t)N);
        mfem::k_pack_mask<<<mfem::blocks_for(N, 256), 256, 0, c.stream>>>(raw, N, d);
        mfem::check_launch("k_pack_mask");
        c.hasMask = true;
    });
}

int mfem_prec_init(mfem_context *ctx) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::require_pattern(c);
        MFEM_REQUIRE(c.lastOp >= 0, MFEM_ERR_STATE, "prec_init before assembly");
        mfem::pipeline_guard(c);
        mfem::prec_init_fp64(c, c.lastOp);
        c.precIsInit = false;
        c.precBlocks = true;
    });
}

int mfem_prec_inversion(mfem_context *ctx, int *nbSingular) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::require_pattern(c);
        MFEM_REQUIRE(c.lastOp >= 0 && c.prec.ptr, MFEM_ERR_STATE, "prec_inversion before prec_init");
        mfem::pipeline_guard(c);
        int s = mfem::prec_invert(c, c.lastOp);
        if (nbSingular) *nbSingular = s;
        c.precIsInit = true;
        c.precBlocks = false;
    });
}

int mfem_set_sliver_threshold(mfem_context *ctx, double threshold) {
    return mfem::guarded(ctx, [&](Context &c) {
        MFEM_REQUIRE(threshold >= 0.0 && threshold <= 1.0, MFEM_ERR_INVALID_ARG,
                     "threshold must lie in [0, 1]");
        c.sliverThreshold = (float)threshold;
    });
}

int mfem_set_option(mfem_context *ctx, const char *name, double value) {
    return mfem::guarded(ctx, [&](Context &c) {
        MFEM_REQUIRE(name, MFEM_ERR_INVALID_ARG, "null option name");
        const std::string n(name);
        if (n == "sliver_threshold") {
            MFEM_REQUIRE(value >= 0.0 && value <= 1.0, MFEM_ERR_INVALID_ARG, "threshold must lie in [0, 1]");
            c.sliverThreshold = (float)value;
        } else if (n == "fp32_kernel") {
            MFEM_REQUIRE(value == 0.0 || value == 1.0, MFEM_ERR_INVALID_ARG, "fp32_kernel is 0 or 1");
            c.fp32Kernel = (int)value;
        } else if (n == "tile_rows") {
            MFEM_REQUIRE(value >= 1 && value <= 1024, MFEM_ERR_INVALID_ARG, "tile_rows in [1, 1024]");
            c.tiles.maxRows = (int)value;
            c.tiles.built = false;
        } else if (n == "wait_limit") {
            MFEM_REQUIRE(value >= 1 && value <= 4294967295.0, MFEM_ERR_INVALID_ARG, "wait_limit >= 1");
            c.waitLimit = (unsigned)value;
        } else if (n == "test_missing_bytes") {
            MFEM_REQUIRE(value >= 0 && value <= 4096 && (long long)value % 16 == 0, MFEM_ERR_INVALID_ARG,
                         "test_missing_bytes: a multiple of 16 in [0, 4096]");
            c.testExtraTx = (unsigned)value;
        } else if (n == "tile_elems") {
            MFEM_REQUIRE(value >= 64 && value <= 4096, MFEM_ERR_INVALID_ARG, "tile_elems in [64, 4096]");
            c.tiles.maxElem = (int)value;
            c.tiles.built = false;
        } else {
            throw Error(MFEM_ERR_INVALID_ARG, "unknown option " + n);
        }
    });
}

int mfem_get_flagged(mfem_context *ctx, int *nbFlagged) {
    return mfem::guarded(ctx, [&](Context &c) {
        MFEM_REQUIRE(nbFlagged, MFEM_ERR_INVALID_ARG, "null out pointer");
        int h[6] = {0, 0, 0, 0, 0, 0};
        mfem::read_status(c, h, 6);
        *nbFlagged = c.flaggedPending ? h[5] : 0;
    });
}

int mfem_get_values(mfem_context *ctx, double *values) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::check_async(c);
        MFEM_REQUIRE(c.lastOp >= 0, MFEM_ERR_STATE, "nothing assembled");
        MFEM_REQUIRE(values, MFEM_ERR_INVALID_ARG, "null values");
        const long long n = (long long)c.nnz * mfem::op_dim(c.lastOp);
        if (c.lastPrecision == MFEM_FP64) {
            MFEM_CUDA(cudaMemcpyAsync(values, c.values.as<double>(), sizeof(double) * n,
                                      cudaMemcpyDeviceToHost, c.stream));
        } else {
            double *tmp = (double *)c.scratch.reserve(sizeof(double) * n);
            mfem::k_f32_to_f64<<<mfem::blocks_for(n, 256), 256, 0, c.stream>>>(c.values.as<float>(), tmp, n);
            mfem::check_launch("k_f32_to_f64");
            MFEM_CUDA(cudaMemcpyAsync(values, tmp, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
        }
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int mfem_get_values_f32(mfem_context *ctx, float *values) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::check_async(c);
        MFEM_REQUIRE(c.lastOp >= 0 && c.lastPrecision == MFEM_FP32, MFEM_ERR_STATE,
                     "no FP32 assembly to read");
        MFEM_REQUIRE(values, MFEM_ERR_INVALID_ARG, "null values");
        const long long n = (long long)c.nnz * mfem::op_dim(c.lastOp);
        MFEM_CUDA(cudaMemcpyAsync(values, c.values.as<float>(), sizeof(float) * n,
                                  cudaMemcpyDeviceToHost, c.stream));
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int mfem_get_prec(mfem_context *ctx, double *prec) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::check_async(c);
        MFEM_REQUIRE(c.lastOp >= 0 && c.prec.ptr, MFEM_ERR_STATE, "no preconditioner");
        MFEM_REQUIRE(prec, MFEM_ERR_INVALID_ARG, "null prec");
        MFEM_CUDA(cudaMemcpyAsync(prec, c.prec.as<double>(),
                                  sizeof(double) * (size_t)c.nbNodes * mfem::op_dim(c.lastOp),
                                  cudaMemcpyDeviceToHost, c.stream));
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int mfem_values_device(mfem_context *ctx, void **values, int *precision) {
    return mfem::guarded(ctx, [&](Context &c) {
        MFEM_REQUIRE(values, MFEM_ERR_INVALID_ARG, "null out pointer");
        *values = c.values.ptr;
        if (precision) *precision = c.lastPrecision;
    });
}

int mfem_prec_device(mfem_context *ctx, double **prec) {
    return mfem::guarded(ctx, [&](Context &c) {
        MFEM_REQUIRE(prec, MFEM_ERR_INVALID_ARG, "null out pointer");
        *prec = c.prec.as<double>();
    });
}

int mfem_synchronize(mfem_context *ctx) {
    return mfem::guarded(ctx, [&](Context &c) { mfem::check_async(c); });
}

int mfem_profile(mfem_context *ctx, int enable) {
    return mfem::guarded(ctx, [&](Context &c) {
        c.timer.on = enable != 0;
        c.timer.reset();
    });
}

int mfem_profile_read(mfem_context *ctx, char *names, int namesCap, float *ms, int cap,
                      int *count) {
    return mfem::guarded(ctx, [&](Context &c) {
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
        const int n = (int)c.timer.used;
        if (count) *count = n;
        std::string all;
        for (int i = 0; i < n && i < cap; i++) {
            float t = 0.f;
            MFEM_CUDA(cudaEventElapsedTime(&t, c.timer.recs[i].a, c.timer.recs[i].b));
            if (ms) ms[i] = t;
            all += c.timer.recs[i].name;
            all += ';';
        }
        if (names && namesCap > 0) {
            std::strncpy(names, all.c_str(), (size_t)namesCap - 1);
            names[namesCap - 1] = 0;
        }
        c.timer.reset();
    });
}

int mfem_get_sizes(mfem_context *ctx, int *nbElem, int *nbNodes, int *nbEdges, int *nbColors) {
    if (!ctx) return MFEM_ERR_INVALID_ARG;
    if (nbElem) *nbElem = ctx->c.nbElem;
    if (nbNodes) *nbNodes = ctx->c.nbNodes;
    if (nbEdges) *nbEdges = ctx->c.hasPattern ? ctx->c.nnz : 0;
    if (nbColors) *nbColors = ctx->c.coloring.built ? ctx->c.coloring.nbColors : 0;
    return MFEM_OK;
}

// ---- reference-shaped calls ---------------------------------------------------

int mfem_assembly(mfem_context *ctx, double *coord, double *nodeToNodeValue, int *nodeToNodeRow,
                  int *nodeToNodeColumn, int *elemToNode, int *elemToEdge, int nbElem,
                  int nbEdges, int operatorDim, int operatorID) {
    (void)elemToEdge;   // positions are derived on the device
    return mfem::guarded(ctx, [&](Context &c) {
        MFEM_REQUIRE(operatorID == MFEM_OP_LAP || operatorID == MFEM_OP_ELA, MFEM_ERR_INVALID_ARG,
                     "operatorID must be 0 or 1");
        MFEM_REQUIRE(operatorDim == mfem::op_dim(operatorID), MFEM_ERR_INVALID_ARG,
                     "operatorDim does not match operatorID");
        MFEM_REQUIRE(coord && nodeToNodeValue && nodeToNodeRow && nodeToNodeColumn && elemToNode,
                     MFEM_ERR_INVALID_ARG, "null argument");
        // the mesh is re-uploaded (and the pattern re-adopted) when elemToNode is
        // another array or the same array with other contents -- e.g. permuted
        // in place as src/main.cc:229 does after coloring_creation
        if (c.nbElem != nbElem || c.hostE2n != elemToNode ||
            c.hostE2nSig != mfem::fingerprint_i32(elemToNode, 4LL * nbElem)) {
            int nbNodes = 0;
            for (long long i = 0; i < 4LL * nbElem; i++) nbNodes = std::max(nbNodes, elemToNode[i]);
            mfem::set_mesh(c, coord, elemToNode, nbElem, nbNodes);
        } else {
            mfem::upload_coords(c, coord);
        }
        if (!c.hasPattern || c.hostRow != nodeToNodeRow || c.hostCol != nodeToNodeColumn ||
            c.nnz != nbEdges) {
            mfem::adopt_pattern(c, nodeToNodeRow, nodeToNodeColumn, nbEdges);
            c.hostRow = nodeToNodeRow;
            c.hostCol = nodeToNodeColumn;
        }
        mfem::assemble(c, operatorID, MFEM_FP64, MFEM_GATHER, false);
        MFEM_CUDA(cudaMemcpyAsync(nodeToNodeValue, c.values.as<double>(),
                                  sizeof(double) * (size_t)nbEdges * operatorDim,
                                  cudaMemcpyDeviceToHost, c.stream));
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int mfem_prec_init_host(mfem_context *ctx, double *prec, double *nodeToNodeValue,
                        int *nodeToNodeRow, int *nodeToNodeColumn, int nbNodes,
                        int operatorDim) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::require_pattern(c);
        MFEM_REQUIRE(prec && nodeToNodeValue, MFEM_ERR_INVALID_ARG, "null argument");
        MFEM_REQUIRE(nbNodes == c.nbNodes, MFEM_ERR_INVALID_ARG, "nbNodes differs from the mesh");
        MFEM_REQUIRE(nodeToNodeRow == c.hostRow && nodeToNodeColumn == c.hostCol, MFEM_ERR_PATTERN,
                     "prec_init on a pattern other than the assembled one");
        const int op = operatorDim == 1 ? MFEM_OP_LAP : MFEM_OP_ELA;
        MFEM_REQUIRE(operatorDim == 1 || operatorDim == 9, MFEM_ERR_INVALID_ARG, "operatorDim must be 1 or 9");
        // the values the caller holds are the source (they may have been changed)
        const size_t n = (size_t)c.nnz * operatorDim;
        mfem::pipeline_guard(c);
        double *dv = (double *)c.values.reserve(sizeof(double) * n);
        MFEM_CUDA(cudaMemcpyAsync(dv, nodeToNodeValue, sizeof(double) * n, cudaMemcpyHostToDevice, c.stream));
        c.lastOp = op;
        c.lastPrecision = MFEM_FP64;
        mfem::prec_init_fp64(c, op);
        c.precIsInit = false;
        c.precBlocks = true;
        MFEM_CUDA(cudaMemcpyAsync(prec, c.prec.as<double>(), sizeof(double) * (size_t)nbNodes * operatorDim,
                                  cudaMemcpyDeviceToHost, c.stream));
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int mfem_prec_inversion_host(mfem_context *ctx, double *prec, int *nodeToNodeRow,
                             int *nodeToNodeColumn, int *checkBounds, int nbNodes,
                             int operatorID) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::require_pattern(c);
        MFEM_REQUIRE(prec, MFEM_ERR_INVALID_ARG, "null prec");
        MFEM_REQUIRE(nbNodes == c.nbNodes, MFEM_ERR_INVALID_ARG, "nbNodes differs from the mesh");
        MFEM_REQUIRE(nodeToNodeRow == c.hostRow && nodeToNodeColumn == c.hostCol, MFEM_ERR_PATTERN,
                     "prec_inversion on a pattern other than the assembled one");
        MFEM_REQUIRE(operatorID == MFEM_OP_LAP || operatorID == MFEM_OP_ELA, MFEM_ERR_INVALID_ARG,
                     "operatorID must be 0 or 1");
        const int dim = mfem::op_dim(operatorID);
        if (operatorID == MFEM_OP_ELA) {
            MFEM_REQUIRE(checkBounds, MFEM_ERR_INVALID_ARG, "null checkBounds");
            const int rc = mfem_set_check_bounds(ctx, checkBounds);
            if (rc != MFEM_OK) throw Error(rc, c.lastError);
        }
        mfem::pipeline_guard(c);
        double *dp = (double *)c.prec.reserve(sizeof(double) * (size_t)nbNodes * dim);
        MFEM_CUDA(cudaMemcpyAsync(dp, prec, sizeof(double) * (size_t)nbNodes * dim,
                                  cudaMemcpyHostToDevice, c.stream));
        mfem::prec_invert(c, operatorID);
        MFEM_CUDA(cudaMemcpyAsync(prec, dp, sizeof(double) * (size_t)nbNodes * dim,
                                  cudaMemcpyDeviceToHost, c.stream));
        MFEM_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int mfem_step_async(mfem_context *ctx, int operatorID, int precision, int strategy,
                    const double *coord, const double *coef, void *values, double *prec,
                    long long *ticket) {
    return mfem::guarded(ctx, [&](Context &c) {
        const long long t = mfem::step_async(c, operatorID, precision, strategy, coord, coef, values, prec);
        if (ticket) *ticket = t;
    });
}

int mfem_wait(mfem_context *ctx, long long ticket) {
    return mfem::guarded(ctx, [&](Context &c) { mfem::wait_step(c, ticket); });
}

int mfem_spmv(mfem_context *ctx, const double *x, double *y, int constrained) {
    return mfem::guarded(ctx, [&](Context &c) {
        MFEM_REQUIRE(x && y, MFEM_ERR_INVALID_ARG, "null vector");
        mfem::spmv_device(c, x, y, constrained);
    });
}

int mfem_prec_apply(mfem_context *ctx, const double *r, double *z) {
    return mfem::guarded(ctx, [&](Context &c) {
        MFEM_REQUIRE(r && z, MFEM_ERR_INVALID_ARG, "null vector");
        mfem::prec_apply_device(c, r, z);
    });
}

int mfem_pcg(mfem_context *ctx, const double *b, double *x, double rtol, int maxIter, int constrained,
             int *iters, double *relres) {
    return mfem::guarded(ctx, [&](Context &c) {
        mfem::check_async(c);
        mfem::pcg(c, b, x, rtol, maxIter, constrained, iters, relres);
    });
}

}  // extern "C"
