/* minifem_dropin.h — the reference's operator signatures, implemented on the
 * GB300 over the C ABI of mfem_gpu.h (mini-fem_gb300/host/operators_gpu.cc).
 *
 * A reference build that compiles operators_gpu.cc instead of
 * src/assembly.cc, src/preconditioner.cc, src/matrix.cc, src/coloring.cc and
 * src/Fortran/elasclpr.f links against these unchanged.  Define
 * MINIFEM_WITH_DC_H to take index_t from the caller's DC-lib header (so the C++
 * names mangle exactly as the reference's declarations); otherwise the layout
 * the reference relies on (index, value) is declared here.
 *
 * Errors: message on stderr and exit(EXIT_FAILURE), as the reference does
 * (src/coloring.cc:66-69, src/IO.cc:33-36).
 */
#ifndef MINIFEM_DROPIN_H
#define MINIFEM_DROPIN_H

#ifdef MINIFEM_WITH_DC_H
#include <DC.h>
#else
typedef struct index_s {
    int *index = nullptr;
    int *value = nullptr;
} index_t;
#endif

/* Globals the reference's driver defines (src/main.cc:44-45), set by
 * coloring_creation (src/headers/globals.h:43-44). */
extern int *colorToElem;
extern int nbTotalColors;

/* src/headers/matrix.h:23-28 */
void create_elemToEdge (int *nodeToNodeRow, int *nodeToNodeColumn, int *elemToNode,
                        int *elemToEdge, int nbElem);
void create_nodeToNode (int *nodeToNodeRow, int *nodeToNodeColumn,
                        index_t &nodeToElem, int *elemToNode, int nbNodes);

/* src/headers/coloring.h:31 */
void coloring_creation (int *elemToNode, int *colorPerm, int nbElem, int nbNodes);

/* src/headers/assembly.h:61-63 (non-MULTITHREADED_COMM form) */
void assembly (double *coord, double *nodeToNodeValue, int *nodeToNodeRow,
               int *nodeToNodeColumn, int *elemToNode, int *elemToEdge, int nbElem,
               int nbEdges, int operatorDim, int operatorID);

/* src/headers/preconditioner.h:27-32 */
void prec_inversion (double *prec, int *nodeToNodeRow, int *nodeToNodeColumn,
                     int *checkBounds, int nbNodes, int operatorID);
void prec_init (double *prec, double *nodeToNodeValue, int *nodeToNodeRow,
                int *nodeToNodeColumn, int nbNodes, int operatorDim);

#endif
