/* Oracle (test infrastructure only): the reference's three Fortran routines with
 * their Fortran-ABI names, restated in C (no Fortran compiler or LAPACK here).
 * They forward to the restatements in oracle.c:
 *   dqmrd4_          src/Fortran/qdmrd4.f:1-23
 *   e_essbcm_        src/Fortran/e_cgmelissa.F:13-47
 *   ela_invert_prec_ src/Fortran/elasclpr.f:2-56 (DGETRF/DGETRI from lapack3.h)
 * The reference prints "!!! info[DGETRF]=" on a singular block and carries on;
 * this stand-in carries on without printing. */
#include "../oracle.h"

void dqmrd4_ (int *nbNodes, int *boundNodesCode, int *nbBoundNodes,
              int *boundNodesList, int *error)
{
    orc_dqmrd4 (*nbNodes, boundNodesCode, nbBoundNodes, boundNodesList, error);
}

void e_essbcm_ (int *dimNode, int *nbNodes, int *nbBoundNodes, int *boundNodesList,
                int *boundNodesCode, int *checkBounds)
{
    orc_e_essbcm (*dimNode, *nbNodes, *nbBoundNodes, boundNodesList, boundNodesCode,
                  checkBounds);
}

void ela_invert_prec_ (int *dimNode, int *nbNodes, int *nodeToNodeIndex,
                       int *nodeToNodeValue, double *prec, int *error,
                       int *checkBounds, int *curNode)
{
    orc_ela_invert_prec (*dimNode, *nbNodes, nodeToNodeIndex, nodeToNodeValue, prec,
                         error, checkBounds, *curNode);
}
