// The reference's operators (src/matrix.cc, src/coloring.cc, src/assembly.cc,
// src/preconditioner.cc) with their own signatures, computed on the GB300
// through the C ABI.  One device context per process, created on first use on
// device $MINIFEM_DEVICE (default 0).
#include <climits>
#include <cstdlib>
#include <iostream>

#include "mfem_gpu.h"
#include "minifem_dropin.h"

namespace {

mfem_context *g_ctx = nullptr;

void die(int rc, const char *where) {
    std::cerr << "Error: " << where << ": " << mfem_status_string(rc) << ": "
              << (g_ctx ? mfem_last_error(g_ctx) : "") << "\n";
    exit(EXIT_FAILURE);
}

void check(int rc, const char *where) {
    if (rc != MFEM_OK) die(rc, where);
}

mfem_context *ctx() {
    if (!g_ctx) {
        const char *d = getenv("MINIFEM_DEVICE");
        check(mfem_create(&g_ctx, d ? atoi(d) : 0), "mfem_create");
    }
    return g_ctx;
}

}  // namespace

void create_nodeToNode(int *nodeToNodeRow, int *nodeToNodeColumn, index_t &nodeToElem,
                       int *elemToNode, int nbNodes) {
    // nodeToElem lists every (node, element) incidence: its last offset is 4 nbElem
    const int nbElem = nodeToElem.index[nbNodes] / 4;
    check(mfem_set_mesh(ctx(), nullptr, elemToNode, nbElem, nbNodes), "create_nodeToNode");
    int nnz = 0;
    // the columns follow the caller's node -> element order, as src/matrix.cc:66-85 does
    check(mfem_create_nodeToNode_incidence(ctx(), nodeToElem.index, nodeToElem.value,
                                           nodeToNodeRow, nodeToNodeColumn, INT_MAX, &nnz),
          "create_nodeToNode");
}

void create_elemToEdge(int *nodeToNodeRow, int *nodeToNodeColumn, int *elemToNode,
                       int *elemToEdge, int nbElem) {
    (void)elemToNode;
    (void)nbElem;
    int nnz = 0;
    check(mfem_get_sizes(ctx(), nullptr, nullptr, &nnz, nullptr), "create_elemToEdge");
    (void)nodeToNodeRow;
    (void)nodeToNodeColumn;
    check(mfem_create_elemToEdge(ctx(), elemToEdge), "create_elemToEdge");
}

void coloring_creation(int *elemToNode, int *colorPerm, int nbElem, int nbNodes) {
    check(mfem_set_mesh(ctx(), nullptr, elemToNode, nbElem, nbNodes), "coloring_creation");
    int index[129], nc = 0;
    check(mfem_coloring_creation(ctx(), 0ULL, colorPerm, index, 129, &nc), "coloring_creation");
    delete[] colorToElem;
    colorToElem = new int[nc + 1];
    for (int c = 0; c <= nc; c++) colorToElem[c] = index[c];
    nbTotalColors = nc;
}

void assembly(double *coord, double *nodeToNodeValue, int *nodeToNodeRow, int *nodeToNodeColumn,
              int *elemToNode, int *elemToEdge, int nbElem, int nbEdges, int operatorDim,
              int operatorID) {
    check(mfem_assembly(ctx(), coord, nodeToNodeValue, nodeToNodeRow, nodeToNodeColumn,
                        elemToNode, elemToEdge, nbElem, nbEdges, operatorDim, operatorID),
          "assembly");
}

void prec_init(double *prec, double *nodeToNodeValue, int *nodeToNodeRow, int *nodeToNodeColumn,
               int nbNodes, int operatorDim) {
    check(mfem_prec_init_host(ctx(), prec, nodeToNodeValue, nodeToNodeRow, nodeToNodeColumn,
                              nbNodes, operatorDim),
          "prec_init");
}

void prec_inversion(double *prec, int *nodeToNodeRow, int *nodeToNodeColumn, int *checkBounds,
                    int nbNodes, int operatorID) {
    check(mfem_prec_inversion_host(ctx(), prec, nodeToNodeRow, nodeToNodeColumn, checkBounds,
                                   nbNodes, operatorID),
          "prec_inversion");
}
