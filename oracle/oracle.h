/* Oracle (test infrastructure only): CPU restatement of Mini-FEM's assembly step.
 *
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark may load
 * this library, and only as the checker / the timed CPU baseline, never as a
 * product path.  Each function names the reference lines it restates.
 *
 * Index conventions follow the reference: elemToNode and CSR columns are
 * 1-based, CSR row pointers are 0-based, element ids are 0-based.
 */
#ifndef MINIFEM_ORACLE_H
#define MINIFEM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Node -> element incidence in ascending element order per node.
 * Restates the contract of DC-lib's DC_create_nodeToElem as used by
 * src/main.cc:243-247 and src/coloring.cc:90-93 (DC-lib itself is absent). */
void orc_node_to_elem(int nbNodes, int nbElem, const int *elemToNode,
                      int *index, int *value);

/* src/matrix.cc:55-91 create_nodeToNode: first-occurrence column order. */
void orc_create_nodeToNode(int *row, int *col, const int *nteIndex,
                           const int *nteValue, const int *elemToNode, int nbNodes);

/* src/matrix.cc:25-52 create_elemToEdge. */
void orc_create_elemToEdge(const int *row, const int *col, const int *elemToNode,
                           int *elemToEdge, int nbElem);

/* src/assembly.cc:615-659 (REF build): zero the values, then assemble every
 * element in ascending order with the row search of assembly.cc:413-421 /
 * :548-554.  coef == NULL gives the reference's fixed operator; otherwise coef
 * holds kappa[nbElem] (lap) or (E, nu)[nbElem*2] (ela), see oracle.c. */
void orc_assembly(const double *coord, double *values, const int *row,
                  const int *col, const int *elemToNode, int nbElem, int nbEdges,
                  int operatorDim, int operatorID, const double *coef);

/* The same arithmetic driven by the reference's OPTIMIZED path
 * (assembly.cc:379-412): positions taken from elemToEdge, no row search. */
void orc_assembly_positions(const double *coord, double *values,
                            const int *elemToEdge, const int *elemToNode,
                            int nbElem, int nbEdges, int operatorDim, int operatorID,
                            const double *coef);

/* Colour-ordered assembly (assembly.cc:593-611, COLORING build): elements are
 * visited colour by colour through order[] (a permutation of element ids) and
 * each colour's elements in the order given. */
void orc_assembly_ordered(const double *coord, double *values, const int *row,
                          const int *col, const int *elemToNode, const int *order,
                          int nbElem, int nbEdges, int operatorDim, int operatorID,
                          const double *coef);

/* src/preconditioner.cc:52-87 prec_init. */
void orc_prec_init(double *prec, const double *values, const int *row,
                   const int *col, int nbNodes, int operatorDim);

/* src/preconditioner.cc:25-49 prec_inversion (+ src/Fortran/elasclpr.f for ela).
 * Returns the number of blocks for which DGETRF/DGETRI reported INFO != 0. */
/* Threads the OpenMP loops use (1 without OpenMP). */
int orc_threads(void);
void orc_halo_pack(const double *prec, const int *intfIndex, const int *intfNodes, int nbIntf,
                   int operatorDim, double *bufferSend);
void orc_halo_add(double *prec, const int *intfIndex, const int *intfNodes, int nbIntf,
                  int operatorDim, const double *bufferRecv);
void orc_set_threads(int n);
int orc_prec_inversion(double *prec, const int *row, const int *col,
                       const int *checkBounds, int nbNodes, int operatorID);

/* src/Fortran/elasclpr.f:2-56 for one node i (1-based). */
void orc_ela_invert_prec(int nspa, int nnt, const int *innv, const int *nnv,
                         double *prec, int *ier, const int *markf, int i);

/* src/Fortran/qdmrd4.f:1-23 and src/Fortran/e_cgmelissa.F:13-47. */
void orc_dqmrd4(int nnt, const int *jlog, int *nnd, int *nlim, int *ier);
void orc_e_essbcm(int ndim, int nbp, int nnd, const int *nlim, const int *jlog,
                  int *markf);

/* src/coloring.cc:27-109: greedy first-fit colouring (<= 128 colours) of the
 * element graph; colorPart[e] = colour; colorToElem[c] = first element of colour
 * c in colour-sorted order.  Returns the number of colours, or -1 when more than
 * 128 would be needed (the reference exits at coloring.cc:66-69). */
int orc_coloring(const int *elemToNode, int nbElem, int nbNodes, int *colorPart,
                 int *colorToElem);

/* Frobenius norm as src/FEM.cc:48-56 computes it. */
double orc_norm(const double *x, long n);

/* 3x3 DGETRF + DGETRI restatement on a column-major block, for direct tests. */
int orc_getrf_getri3(double *a);

#ifdef __cplusplus
}
#endif
#endif
