// Allocation-free FP64 assembly (mfem_assemble_noalloc).
//
// Some callers cannot call cudaMalloc while they assemble: solvers whose device
// memory is owned by their own pool allocator and that forbid other allocations
// after start-up, time-stepping loops that must not stall on cudaFree's implicit
// device synchronisation, and real-time loops that must not take the
// allocator's locks or risk an out-of-memory failure mid-run.  This
// entry point runs the FP64 gather -- the same kernels as mfem_assemble with
// MFEM_FP64 / MFEM_GATHER -- on buffers the caller passes (coordinates,
// coefficients, values) and keeps its only scratch, the per-element gradient
// records, in the file-scope array below instead of allocating it.
#include <mutex>

#include "context.h"
#include "elem_math.cuh"

namespace mfem {
void gather_fp64_into(const Context &c, int op, const double *coord, const double *coef,
                      double *rec, double *values, cudaStream_t s);
}

namespace {

// Largest mesh the allocation-free entry point accepts: 131,072 elements, i.e.
// 16 MiB of gradient records (128 bytes per element).  Every GPU that loads the
// library holds this array until the process exits.
constexpr int kNoAllocMaxElem = 131072;

static __device__ __align__(256) double g_noalloc_rec[(size_t)kNoAllocMaxElem * mfem::kRec64];

// Device address of g_noalloc_rec for each device, looked up once per device.
// In host code the name g_noalloc_rec is only a host-side stand-in for the
// symbol, never a device address, so kernels get this pointer instead.
std::mutex g_mutex;
constexpr int kMaxDevices = 64;
double *g_rec_addr[kMaxDevices] = {};

// Makes `device` current for the scope and gives the caller's current device
// back on every exit path, so the entry point leaves the calling thread's
// device setting as it found it.
struct DeviceScope {
    int saved = -1;
    explicit DeviceScope(int device) {
        MFEM_CUDA(cudaGetDevice(&saved));
        if (saved != device) MFEM_CUDA(cudaSetDevice(device));
    }
    ~DeviceScope() {
        int now = -1;
        if (saved >= 0 && cudaGetDevice(&now) == cudaSuccess && now != saved) cudaSetDevice(saved);
    }
    DeviceScope(const DeviceScope &) = delete;
    DeviceScope &operator=(const DeviceScope &) = delete;
};

// Called with `device` current (DeviceScope).
double *scratch_address(int device) {
    MFEM_REQUIRE(device >= 0 && device < kMaxDevices, MFEM_ERR_INVALID_ARG, "device id out of range");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_rec_addr[device]) {
        void *p = nullptr;
        const cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_rec);
        if (rc != cudaSuccess)
            throw mfem::Error(MFEM_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_rec): ") +
                                                 cudaGetErrorString(rc));
        g_rec_addr[device] = static_cast<double *>(p);
    }
    return g_rec_addr[device];
}

}  // namespace

extern "C" int mfem_assemble_noalloc(mfem_context *ctx, int operatorID, const double *coord,
                                     const double *coef, double *values, void *stream) {
    if (!ctx) return MFEM_ERR_INVALID_ARG;
    mfem::Context &c = ctx->c;
    try {
        MFEM_REQUIRE(operatorID == MFEM_OP_LAP || operatorID == MFEM_OP_ELA, MFEM_ERR_INVALID_ARG,
                     "operatorID must be 0 or 1");
        MFEM_REQUIRE(coord && values, MFEM_ERR_INVALID_ARG, "null coord or values");
        MFEM_REQUIRE(c.hasPattern && c.gather.built, MFEM_ERR_STATE,
                     "no gather plan: call mfem_assemble(FP64, GATHER) once first");
        MFEM_REQUIRE(c.nbElem <= kNoAllocMaxElem, MFEM_ERR_CAPACITY,
                     "mesh larger than the 131072 elements of the allocation-free scratch");
        DeviceScope scope(c.device);
        if (stream) {
            int sdev = -1;
            MFEM_CUDA(cudaStreamGetDevice((cudaStream_t)stream, &sdev));
            MFEM_REQUIRE(sdev == c.device, MFEM_ERR_INVALID_ARG,
                         "stream belongs to another device than the context");
        }
        double *rec = scratch_address(c.device);
        mfem::gather_fp64_into(c, operatorID, coord, coef, rec, values, (cudaStream_t)stream);
        c.lastError.clear();
        return MFEM_OK;
    } catch (const mfem::Error &e) {
        c.lastError = e.what();
        return e.code;
    }
}
