/* Oracle (test infrastructure only): C entry points over the reference's own
 * C++ operators, compiled together with the reference sources by the Makefile
 * in this folder (outputs in _ref/, never committed).  Tests load the result
 * with ctypes to pin the CPU restatement (oracle.c) against the reference:
 *   ref_create_pattern  -> DC_create_nodeToElem + create_nodeToNode
 *                          (src/main.cc:243-250, src/matrix.cc:55-91)
 *   ref_create_elemToEdge -> create_elemToEdge (src/matrix.cc:25-52)
 *   ref_assembly        -> assembly (src/assembly.cc:615-720)
 *   ref_prec_init       -> prec_init (src/preconditioner.cc:52-87)
 *   ref_prec_inversion  -> prec_inversion (src/preconditioner.cc:25-49)
 *   ref_coloring        -> coloring_creation + DC_permute_int_2d_array
 *                          (src/coloring.cc:84-109, src/main.cc:216-230)
 * The build flavour (-DREF or -DCOLORING) decides which variant these run. */
#include <string>

#include "globals.h"
#include "matrix.h"
#include "coloring.h"
#include "assembly.h"
#include "preconditioner.h"

/* Globals that src/main.cc:43-45 defines for the driver. */
string meshName, operatorName;
int *colorToElem = nullptr;
int nbTotalColors = 0;

extern "C" {

int ref_create_pattern (int nbNodes, int nbElem, int *elemToNode, int *row, int *col)
{
    index_t nodeToElem;
    nodeToElem.index = new int [nbNodes + 1];
    nodeToElem.value = new int [(long)nbElem * DIM_ELEM];
    DC_create_nodeToElem (nodeToElem, elemToNode, nbElem, DIM_ELEM, nbNodes);
    create_nodeToNode (row, col, nodeToElem, elemToNode, nbNodes);
    delete[] nodeToElem.value;
    delete[] nodeToElem.index;
    return row[nbNodes];
}

void ref_create_elemToEdge (int *row, int *col, int *elemToNode, int *elemToEdge,
                            int nbElem)
{
    create_elemToEdge (row, col, elemToNode, elemToEdge, nbElem);
}

void ref_assembly (double *coord, double *values, int *row, int *col, int *elemToNode,
                   int nbElem, int nbEdges, int operatorDim, int operatorID)
{
    assembly (coord, values, row, col, elemToNode, nullptr, nbElem, nbEdges,
              operatorDim, operatorID);
}

void ref_prec_init (double *prec, double *values, int *row, int *col, int nbNodes,
                    int operatorDim)
{
    prec_init (prec, values, row, col, nbNodes, operatorDim);
}

void ref_prec_inversion (double *prec, int *row, int *col, int *checkBounds,
                         int nbNodes, int operatorID)
{
    prec_inversion (prec, row, col, checkBounds, nbNodes, operatorID);
}

/* Colours the mesh and permutes elemToNode in place into colour order, as the
 * COLORING driver does, and keeps the colour index set for a following
 * ref_assembly of the COLORING build.  colorIndex receives nbColors+1 offsets. */
int ref_coloring (int *elemToNode, int nbElem, int nbNodes, int *colorPerm,
                  int *colorIndex)
{
    delete[] colorToElem;
    colorToElem = nullptr;
    coloring_creation (elemToNode, colorPerm, nbElem, nbNodes);
    DC_permute_int_2d_array (elemToNode, colorPerm, nbElem, DIM_ELEM, 0);
    for (int c = 0; c <= nbTotalColors; c++) colorIndex[c] = colorToElem[c];
    return nbTotalColors;
}

}
