// Interface-node sum of the preconditioner blocks between sub-domains: the
// device form of MPI_halo_exchange (src/halo.cc:39-122), the one exchange step
// of the reference's domain decomposition (called between prec_init and
// prec_inversion, src/FEM.cc:211-222).
//
// Each rank holds its own sub-domain; interface i lists the local nodes it
// shares with neighbour neighborsList[i] (intfNodes[intfIndex[i] ..
// intfIndex[i+1]), 1-based, the same nodes in the same order on both sides).
// The reference packs every listed node's block into a send buffer
// (src/halo.cc:66-77, from the blocks before any addition), sends interface i's
// slice to its neighbour, receives the neighbour's slice into the same place
// of a receive buffer, and adds the received blocks to its own, interface by
// interface and entry by entry (src/halo.cc:96-112).  Here:
//
//   mfem_halo_pack  -- one kernel gathers the listed blocks into a device send
//                      buffer (same layout as the reference's bufferSend);
//   (the caller moves each interface's slice to its neighbour: NCCL/MPI/gloo
//    send-receive, or any copy; the library does not communicate)
//   mfem_halo_add   -- one thread per (distinct interface node, block value)
//                      adds that node's received values in interface order,
//                      the order of the reference's loop, so a node shared with
//                      several neighbours gets the same bits as the reference.
#include <algorithm>
#include <numeric>
#include <vector>

#include "context.h"

namespace mfem {
namespace {

__global__ void k_halo_pack(const double *__restrict__ prec, const int *__restrict__ node,
                            long long n, int dim, double *__restrict__ send) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long j = i / dim;
    const int k = (int)(i - j * dim);
    send[i] = prec[(size_t)node[j] * dim + k];
}

__global__ void k_halo_add(double *__restrict__ prec, const int *__restrict__ uniqNode,
                           const int *__restrict__ uniqStart, const int *__restrict__ uniqEntry,
                           long long n, int dim, const double *__restrict__ recv) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const long long u = i / dim;
    const int k = (int)(i - u * dim);
    double *p = prec + (size_t)uniqNode[u] * dim + k;
    double acc = *p;
    for (int q = uniqStart[u]; q < uniqStart[u + 1]; q++) acc = acc + recv[(size_t)uniqEntry[q] * dim + k];
    *p = acc;
}

int prec_dim(const Context &c) { return c.lastOp == MFEM_OP_LAP ? 1 : 9; }

void require_blocks(const Context &c) {
    MFEM_REQUIRE(c.halo.built, MFEM_ERR_STATE, "no interfaces (mfem_set_interfaces first)");
    MFEM_REQUIRE(c.precBlocks && c.prec.ptr, MFEM_ERR_STATE,
                 "the halo sum needs the preconditioner blocks of the latest assembly "
                 "before inversion (mfem_prec_init first)");
}

}  // namespace
}  // namespace mfem

using mfem::Context;

extern "C" {

int mfem_set_interfaces(mfem_context *ctx, int nbIntf, const int *intfIndex, const int *intfNodes) {
    return mfem::run_guarded(ctx, [&](Context &c) {
        MFEM_REQUIRE(c.nbNodes > 0, MFEM_ERR_STATE, "no mesh set");
        MFEM_REQUIRE(nbIntf >= 0, MFEM_ERR_INVALID_ARG, "negative nbIntf");
        MFEM_REQUIRE(nbIntf == 0 || intfIndex, MFEM_ERR_INVALID_ARG, "null intfIndex");
        const int m = nbIntf ? intfIndex[nbIntf] : 0;
        MFEM_REQUIRE(nbIntf == 0 || intfIndex[0] == 0, MFEM_ERR_INVALID_ARG, "intfIndex[0] must be 0");
        for (int i = 0; i < nbIntf; i++)
            MFEM_REQUIRE(intfIndex[i + 1] >= intfIndex[i], MFEM_ERR_INVALID_ARG,
                         "intfIndex must be non-decreasing");
        MFEM_REQUIRE(m == 0 || intfNodes, MFEM_ERR_INVALID_ARG, "null intfNodes");
        std::vector<int> node(m);
        for (int j = 0; j < m; j++) {
            MFEM_REQUIRE(intfNodes[j] >= 1 && intfNodes[j] <= c.nbNodes, MFEM_ERR_INVALID_ARG,
                         "intfNodes holds a node outside [1, nbNodes]");
            node[j] = intfNodes[j] - 1;
        }
        // distinct nodes; each node's entries in ascending entry index, which is
        // interface order (entries of interface i precede those of i + 1)
        std::vector<int> order(m);
        std::iota(order.begin(), order.end(), 0);
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return node[a] < node[b]; });
        std::vector<int> uniq, start;
        for (int q = 0; q < m; q++) {
            if (q == 0 || node[order[q]] != node[order[q - 1]]) {
                uniq.push_back(node[order[q]]);
                start.push_back(q);
            }
        }
        start.push_back(m);
        auto up = [&](mfem::DevBuf &b, const std::vector<int> &v) {
            int *d = (int *)b.reserve(sizeof(int) * std::max<size_t>(v.size(), 1));
            if (!v.empty())
                MFEM_CUDA(cudaMemcpyAsync(d, v.data(), sizeof(int) * v.size(), cudaMemcpyHostToDevice,
                                          c.stream));
        };
        up(c.halo.node, node);
        up(c.halo.uniqNode, uniq);
        up(c.halo.uniqStart, start);
        up(c.halo.uniqEntry, order);
        MFEM_CUDA(cudaStreamSynchronize(c.stream));   // the host vectors go out of scope
        c.halo.nbIntf = nbIntf;
        c.halo.nbIntfNodes = m;
        c.halo.nUniq = (int)uniq.size();
        c.halo.built = true;
    });
}

int mfem_halo_pack(mfem_context *ctx, double *sendDevice) {
    return mfem::run_guarded(ctx, [&](Context &c) {
        mfem::require_blocks(c);
        const int dim = mfem::prec_dim(c);
        const long long n = (long long)c.halo.nbIntfNodes * dim;
        if (n == 0) return;
        MFEM_REQUIRE(sendDevice, MFEM_ERR_INVALID_ARG, "null send buffer");
        c.timer.begin("halo_pack", c.stream);
        mfem::k_halo_pack<<<mfem::blocks_for(n, 256), 256, 0, c.stream>>>(
            c.prec.as<double>(), c.halo.node.as<int>(), n, dim, sendDevice);
        mfem::check_launch("k_halo_pack");
        c.timer.end(c.stream);
    });
}

int mfem_halo_add(mfem_context *ctx, const double *recvDevice) {
    return mfem::run_guarded(ctx, [&](Context &c) {
        mfem::require_blocks(c);
        const int dim = mfem::prec_dim(c);
        const long long n = (long long)c.halo.nUniq * dim;
        if (n == 0) return;
        MFEM_REQUIRE(recvDevice, MFEM_ERR_INVALID_ARG, "null receive buffer");
        c.timer.begin("halo_add", c.stream);
        mfem::k_halo_add<<<mfem::blocks_for(n, 256), 256, 0, c.stream>>>(
            c.prec.as<double>(), c.halo.uniqNode.as<int>(), c.halo.uniqStart.as<int>(),
            c.halo.uniqEntry.as<int>(), n, dim, recvDevice);
        mfem::check_launch("k_halo_add");
        c.timer.end(c.stream);
    });
}

}  // extern "C"
