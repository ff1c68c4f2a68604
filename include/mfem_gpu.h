/* mfem_gpu.h — C ABI of the GB300 (sm_103a) implementation of Mini-FEM's
 * assembly step: CSR pattern, element colouring, Laplacian / 3-DOF elasticity
 * assembly of P1 tetrahedra and block-Jacobi preconditioner creation.
 *
 * Plain C types only (pointers and sizes); every function returns an int status
 * (MFEM_OK = 0, negative on failure; mfem_last_error() gives the message).
 * Index conventions are the reference's: elemToNode and CSR columns 1-based,
 * CSR row pointers 0-based (src/matrix.cc:55-91, src/main.cc:243-249).
 * Unless a name ends in _device, pointer arguments are HOST memory.
 *
 * Each entry point names the reference interface it replaces.  The reference
 * operators return void and exit(EXIT_FAILURE) on error
 * (src/coloring.cc:66-69, src/IO.cc:33-36); here the status is returned and the
 * caller decides (include/minifem_dropin.h keeps the exit behaviour).
 */
#ifndef MFEM_GPU_H
#define MFEM_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define MFEM_ABI_VERSION 1

/* status codes */
#define MFEM_OK               0
#define MFEM_ERR_INVALID_ARG (-1)
#define MFEM_ERR_CUDA        (-2)
#define MFEM_ERR_NO_DEVICE   (-3)
#define MFEM_ERR_STATE       (-4)  /* call out of order (e.g. assemble before a mesh) */
#define MFEM_ERR_PATTERN     (-5)  /* nbEdges / pattern mismatch, row too long */
#define MFEM_ERR_COLORS      (-6)  /* more than 128 colours (src/coloring.cc:66-69) */
#define MFEM_ERR_CAPACITY    (-7)  /* caller buffer or fixed limit too small */
#define MFEM_ERR_TIMEOUT     (-8)  /* a bounded device wait gave up */

/* operatorID (src/main.cc:131-138) */
#define MFEM_OP_LAP 0
#define MFEM_OP_ELA 1

/* precision */
#define MFEM_FP64 0   /* FP64 arithmetic and values */
#define MFEM_FP32 1   /* FP32 element arithmetic and values, compensated sums,
                         FP64 for flagged slivers and the block inversion */

/* strategy */
#define MFEM_AUTO    (-1)
#define MFEM_GATHER    0  /* owner-computes, ascending element order (bit-exact FP64) */
#define MFEM_SCATTER   1  /* colour-ordered scatter, no atomics */
#define MFEM_ATOMIC    2  /* element-parallel atomics (order not deterministic) */

/* column order of the CSR pattern */
#define MFEM_ORDER_SORTED    0  /* ascending columns in each row */
#define MFEM_ORDER_REFERENCE 1  /* first occurrence, as src/matrix.cc:55-91 */

typedef struct mfem_context mfem_context;

/* ---- lifecycle ------------------------------------------------------------ */
int mfem_create(mfem_context **ctx, int device);
int mfem_destroy(mfem_context *ctx);
const char *mfem_last_error(const mfem_context *ctx);
const char *mfem_status_string(int status);
int mfem_abi_version(void);
/* The CUDA stream every call of this context is ordered on (cudaStream_t).  A
 * call may fan independent kernels out to a second stream of the context (the
 * FP64 gather's diagonal and off-diagonal units), always joined back to this
 * stream before the call returns: work enqueued on it afterwards, or a wait on
 * it, sees the call complete. */
int mfem_get_stream(mfem_context *ctx, void **stream);

/* ---- mesh (src/IO.cc:61-96 arrays) ----------------------------------------- */
/* Uploads coord[nbNodes*3] and elemToNode[nbElem*4] (1-based).  Replaces the
 * mesh and drops every structure built on the previous one.  coord may be NULL
 * (topology only, as create_nodeToNode sees the mesh); assembly then needs
 * mfem_update_coords first. */
int mfem_set_mesh(mfem_context *ctx, const double *coord, const int *elemToNode,
                  int nbElem, int nbNodes);
/* New coordinates for the same topology (keeps pattern, colouring, plans). */
int mfem_update_coords(mfem_context *ctx, const double *coord);

/* ---- CSR pattern: replaces create_nodeToNode (src/matrix.cc:55-91, called at
 * src/main.cc:247-249) and create_elemToEdge (src/matrix.cc:25-52). ---------- */
/* Builds the pattern on the device.  row[nbNodes+1] and col[capacity] may be
 * NULL (device-only).  *nbEdges receives nnz.  MFEM_ERR_CAPACITY if
 * capacity < nnz (nothing written to col then). */
int mfem_create_nodeToNode(mfem_context *ctx, int order, int *row, int *col,
                           int capacity, int *nbEdges);
/* create_nodeToNode exactly as src/matrix.cc:55-91 computes it from the
 * caller's node -> element lists (index_t nodeToElem of src/main.cc:243-247:
 * index[nbNodes+1], value[index[nbNodes]] = 0-based element ids): the columns of
 * row i are the distinct nodes of the elements value[index[i] .. index[i+1]) in
 * first-occurrence order, walking the lists in the caller's order (the order
 * DC-lib produced).  Other arguments as mfem_create_nodeToNode with
 * MFEM_ORDER_REFERENCE. */
int mfem_create_nodeToNode_incidence(mfem_context *ctx, const int *nodeToElemIndex,
                                     const int *nodeToElemValue, int *row, int *col,
                                     int capacity, int *nbEdges);
/* elemToEdge[nbElem*16]: 0-based CSR position of (j,k), j-major. */
int mfem_create_elemToEdge(mfem_context *ctx, int *elemToEdge);
/* Adopts a pattern the caller built (row 0-based, col 1-based, any column order).
 * Every element pair must be present: MFEM_ERR_PATTERN otherwise. */
int mfem_set_pattern(mfem_context *ctx, const int *row, const int *col, int nbEdges);

/* ---- colouring: replaces coloring_creation (src/coloring.cc:84-109) --------- */
/* Jones-Plassmann first-fit colouring of the element graph on the device
 * (elements sharing a node get different colours), at most 128 colours.
 * colorPerm[nbElem] (may be NULL): colorPerm[old] = position in colour order
 * (stable), the convention src/main.cc:229 applies; colorIndex[nbColors+1]
 * (may be NULL, capacity entries).  The colouring is used by MFEM_SCATTER. */
int mfem_coloring_creation(mfem_context *ctx, unsigned long long seed, int *colorPerm,
                           int *colorIndex, int capacity, int *nbColors);

/* ---- node renumbering (no counterpart in the reference; it orders for locality
 * with DC-lib's D&C permutations, src/main.cc:155-206) ------------------------ */
/* Reverse Cuthill-McKee order of the current pattern's graph:
 * newOfOld[nbNodes], a permutation.  The caller renumbers coord and elemToNode
 * with it and sets the renumbered mesh. */
int mfem_rcm_permutation(mfem_context *ctx, int *newOfOld);
/* Locality orderings of the nodes from the coordinates (newOfOld as above):
 * MFEM_LOCALITY_MORTON -- Z-order of the coordinates (21 bits per axis);
 * MFEM_LOCALITY_BISECTION -- recursive coordinate bisection at the median of
 * the longest axis, leaves of at most 64 nodes numbered depth first: the
 * geometric counterpart of the reference's D&C tree ordering
 * (src/main.cc:155-206, DC-lib).  Renumbering candidates for the tuner beside
 * identity and reverse Cuthill-McKee. */
#define MFEM_LOCALITY_MORTON    1
#define MFEM_LOCALITY_BISECTION 2
int mfem_locality_permutation(mfem_context *ctx, int kind, int *newOfOld);

/* ---- assembly: replaces assembly (src/assembly.cc:615-720) ------------------ */
/* coef == NULL: the reference operator (constants 1 / 2.25, 1.25).  Otherwise
 * lap: kappa[nbElem]; ela: (E, nu)[nbElem*2], Young's modulus and Poisson ratio
 * per element, weighted as lambda = E nu / ((1+nu)(1-2nu)), mu = E / (2(1+nu)). */
int mfem_set_coefficients(mfem_context *ctx, int operatorID, const double *coef);
/* Assembles nodeToNodeValue on the device (kept there).  Enqueued on the
 * context stream; returns without waiting. */
int mfem_assemble(mfem_context *ctx, int operatorID, int precision, int strategy);

/* ---- preconditioner: replaces prec_init (src/preconditioner.cc:52-87) and
 * prec_inversion (src/preconditioner.cc:25-49, src/Fortran/elasclpr.f). ------ */
/* checkBounds[nbNodes*3], column-major MARKF(nbNodes,3) as e_essbcm_ builds it
 * (src/main.cc:340-346).  NULL means no Dirichlet DOF. */
int mfem_set_check_bounds(mfem_context *ctx, const int *checkBounds);
int mfem_prec_init(mfem_context *ctx);
/* *nbSingular (may be NULL) receives the number of blocks whose LU hit an exact
 * zero pivot (the reference prints "info[DGETRF]" and carries on). Synchronises. */
int mfem_prec_inversion(mfem_context *ctx, int *nbSingular);
/* assembly + prec_init + prec_inversion in one enqueue (prec fused into the
 * assembly kernels where the strategy allows). */
int mfem_assemble_prec(mfem_context *ctx, int operatorID, int precision, int strategy);

/* ---- halo: replaces MPI_halo_exchange (src/halo.cc:39-122), the sum of the
 * interface nodes' preconditioner blocks between sub-domains, called between
 * prec_init and prec_inversion (src/FEM.cc:211-222). ------------------------ */
/* The rank's interfaces as src/IO.cc:81-92 reads them: interface i holds the
 * 1-based local nodes intfNodes[intfIndex[i] .. intfIndex[i+1]), listed in the
 * same order on both sides.  nbIntf == 0: a single domain (the sum is a
 * no-op, src/halo.cc:44). */
int mfem_set_interfaces(mfem_context *ctx, int nbIntf, const int *intfIndex,
                        const int *intfNodes);
/* After mfem_prec_init: send[j*opDim + k] = prec block value k of entry j's
 * node (the reference's bufferSend, src/halo.cc:66-77), a DEVICE buffer of
 * intfIndex[nbIntf]*opDim doubles, enqueued on the context stream.  The caller
 * moves slice i (entries intfIndex[i] .. intfIndex[i+1]) to neighbour i and
 * receives the neighbour's slice into the same place of a receive buffer. */
int mfem_halo_pack(mfem_context *ctx, double *sendDevice);
/* prec[node] += recv[entry] for every entry, entries of a node added in
 * interface order (src/halo.cc:96-112): the reference's bits.  recv is a
 * DEVICE buffer laid out as the send buffer; enqueued on the context stream.
 * mfem_prec_inversion follows. */
int mfem_halo_add(mfem_context *ctx, const double *recvDevice);

/* FP32 precision: elements whose shape quality |6V| / (|a| |b| |c|) (a, b, c the
 * edge vectors from the fourth node) is below `threshold` are integrated in FP64
 * (default 0.1).  *nbFlagged receives the count of the last FP32 assembly. */
int mfem_set_sliver_threshold(mfem_context *ctx, double threshold);
int mfem_get_flagged(mfem_context *ctx, int *nbFlagged);
/* Tuning knobs (no counterpart in the reference): "sliver_threshold" (as above),
 * "fp32_kernel" (0: per-element gradient records + one thread per entry,
 * 1: spatial row tiles with gradients in shared memory, the default),
 * "tile_rows" / "tile_elems" (tile size limits of kernel 1), "wait_limit" (polls
 * of the kernel's bounded wait for its staged copies before it gives up and the
 * next result read returns MFEM_ERR_TIMEOUT) and "test_missing_bytes" (testing
 * the bounded wait only: the wait expects that many bytes more than arrive). */
int mfem_set_option(mfem_context *ctx, const char *name, double value);
/* Statistics of the FP32 tile plan (built on demand): tiles, elements over all
 * tiles (halo included), off-diagonal units, contributions, shared memory per
 * CTA in bytes. */
int mfem_tile_info(mfem_context *ctx, int *nbTiles, long long *nbTileElems,
                   long long *nbUnits, long long *nbContrib, int *smemBytes);

/* ---- results ---------------------------------------------------------------- */
int mfem_get_values(mfem_context *ctx, double *values);     /* nbEdges*opDim, FP64 */
int mfem_get_values_f32(mfem_context *ctx, float *values);  /* FP32 assembly only */
int mfem_get_prec(mfem_context *ctx, double *prec);         /* nbNodes*opDim */
/* Device addresses of the results (valid until the next mesh/pattern change). */
int mfem_values_device(mfem_context *ctx, void **values, int *precision);
int mfem_prec_device(mfem_context *ctx, double **prec);
int mfem_synchronize(mfem_context *ctx);
/* Per-kernel timing with CUDA events on the context stream (no counterpart in
 * the reference, whose DC_timer brackets whole steps, src/FEM.cc:182-233).
 * mfem_profile_read synchronises, returns the named regions recorded since
 * the last read ("name;name;..." in names) with their durations in ms, and
 * clears the list. */
int mfem_profile(mfem_context *ctx, int enable);
int mfem_profile_read(mfem_context *ctx, char *names, int namesCap, float *ms, int cap,
                      int *count);
/* Sizes: nbElem, nbNodes, nbEdges, nbColors (any pointer may be NULL). */
int mfem_get_sizes(mfem_context *ctx, int *nbElem, int *nbNodes, int *nbEdges,
                   int *nbColors);

/* ---- pipelined steps ---------------------------------------------------------- */
/* One iteration of the reference's FEM loop (src/FEM.cc:177-234: assembly,
 * prec_init, prec_inversion) with host inputs and host outputs, pipelined: no
 * reference counterpart (its loop is synchronous).  Copies the step's inputs in
 * (coord: nbNodes*3, coef: as mfem_set_coefficients; NULL keeps the current
 * ones), assembles (and, with prec != NULL, the preconditioner) into one of two
 * device result slots, and starts copying the results out into values
 * (nbEdges*opDim floats for MFEM_FP32, doubles for MFEM_FP64) and prec
 * (nbNodes*opDim doubles) on a second stream, then returns a ticket without
 * waiting.  So the copy-out of step k overlaps the copy-in and the assembly of
 * step k+1; a step only waits, on the device, for the copy-out of the step two
 * before it (same slot).  The host buffers of a step must stay untouched until
 * mfem_wait(ticket) returns; page-locked (pinned) buffers make the copies
 * asynchronous.  mfem_wait reports a bounded-wait timeout of that step as
 * MFEM_ERR_TIMEOUT; wait for tickets in order (a slot is reused every two
 * steps).  After mfem_wait the synchronous getters read the latest step. */
int mfem_step_async(mfem_context *ctx, int operatorID, int precision, int strategy,
                    const double *coord, const double *coef, void *values, double *prec,
                    long long *ticket);
int mfem_wait(mfem_context *ctx, long long ticket);

/* ---- consumer of the assembled system ------------------------------------------ */
/* No counterpart in the reference, whose driver names the step after assembly
 * ("assembly, solver & update", src/main.cc:353) without implementing it.  All
 * three use the latest assembly of the context (FP64 or FP32 values; FP64
 * vectors and arithmetic).  constrained != 0 applies the check bounds as
 * homogeneous Dirichlet constraints: a constrained DOF is taken as 0 in every
 * product and its row is the identity (the operator M A M + I - M, whose
 * block-Jacobi inverse is the masked, inverted diagonal block that
 * prec_inversion builds, src/Fortran/elasclpr.f:19-27). */
/* y = A x; x and y are DEVICE pointers (nbNodes*opDim doubles), enqueued on the
 * context stream.  FP64 values: an FP64 FMA chain per row.  FP32 values: x
 * scaled by a power of two and split into two FP32 parts, the products with the
 * high part exact, all summed in double-float, within 15 x 2^-48 of the row's
 * sum of |a x| (measured on random rows of up to 40 blocks); rows
 * the split cannot serve (entries below 2^-60 of max |x|, non-finite values)
 * take the FP64 chain. */
int mfem_spmv(mfem_context *ctx, const double *x, double *y, int constrained);
/* z = P r with the block-Jacobi preconditioner; DEVICE pointers. */
int mfem_prec_apply(mfem_context *ctx, const double *r, double *z);
/* Solves A x = b by conjugate gradients with the block-Jacobi preconditioner
 * until ||b - A x|| <= rtol ||b|| or maxIter iterations; b and x are HOST
 * arrays (x: initial guess in, solution out).  Reductions run in a fixed order:
 * the same inputs give the same bits.  iters, relres (may be NULL): iterations
 * done and the final relative residual of the recurrence. */
int mfem_pcg(mfem_context *ctx, const double *b, double *x, double rtol, int maxIter,
             int constrained, int *iters, double *relres);

/* ---- allocation-free assembly ------------------------------------------------ */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory while they assemble -- solvers whose device memory belongs to their
 * own pool allocator, time-stepping loops that must not stall on cudaFree's
 * implicit device synchronisation, real-time loops that must not risk an
 * allocation failure -- this runs the
 * FP64 gather (the kernels and results of mfem_assemble with MFEM_FP64 and
 * MFEM_GATHER, without the preconditioner) and calls no cudaMalloc, cudaFree or
 * allocating library routine.  coord (nbNodes*3), coef (as
 * mfem_set_coefficients, or NULL for the reference constants) and values
 * (nbEdges*opDim) are DEVICE pointers the caller owns; topology and gather plan
 * are the context's (mfem_assemble with MFEM_FP64/MFEM_GATHER must have run once).
 * Its scratch is one fixed array inside the library of at most 131072 elements
 * (16 MiB of gradient records), held by every GPU that loads the library until
 * the process exits; larger meshes get MFEM_ERR_CAPACITY.  The first call on a
 * device looks the array's device address up (a runtime query that may load
 * the module holding it and synchronise).  Work is enqueued on
 * `stream` (a cudaStream_t, NULL for the legacy default stream) without waiting.
 * All calls share the one array and every call overwrites it: calls that overlap
 * on the GPU (e.g. on two streams) race and must be serialised by the caller.
 * The kernels also read the context's topology and gather plan on `stream`,
 * which is not ordered with the context's own stream: drain `stream` (or make
 * the context stream wait for it) before mfem_set_mesh, mfem_create_nodeToNode,
 * mfem_set_pattern or mfem_destroy change or free them.  The calling thread's
 * current device is left as it was; `stream` must belong to the context's
 * device (MFEM_ERR_INVALID_ARG otherwise). */
int mfem_assemble_noalloc(mfem_context *ctx, int operatorID, const double *coord,
                          const double *coef, double *values, void *stream);

/* ---- batched assembly (no counterpart in the reference, which assembles one
 * mesh per rank, src/FEM.cc:177-257) ------------------------------------------ */
/* Many meshes (contexts with mesh, pattern and Dirichlet mask set; they must not
 * change while in the batch), each with nbSets coefficient sets, assembled per
 * iteration by one CUDA-graph replay: FP32 as ONE persistent launch over a
 * cross-mesh work list of tiles, FP64 as the per-mesh, per-set gather launches.
 * coefSets holds nbSets consecutive per-element arrays laid out as for
 * mfem_set_coefficients (NULL only when nbSets == 1: reference constants). */
typedef struct mfem_batch mfem_batch;
int mfem_batch_create(mfem_batch **batch, int device);
int mfem_batch_destroy(mfem_batch *batch);
const char *mfem_batch_last_error(const mfem_batch *batch);
int mfem_batch_get_stream(mfem_batch *batch, void **stream);
int mfem_batch_add(mfem_batch *batch, mfem_context *ctx, int operatorID, int nbSets,
                   const double *coefSets);
/* New coefficients for item `item` (same layout and count as when added). */
int mfem_batch_set_coefficients(mfem_batch *batch, int item, const double *coefSets);
/* Enqueues one iteration (values of every set; the preconditioner too when
 * withPrec != 0) on the batch stream.  mfem_batch_synchronize waits for it. */
int mfem_batch_assemble(mfem_batch *batch, int precision, int withPrec);
int mfem_batch_synchronize(mfem_batch *batch);
/* values: nbEdges*opDim floats (MFEM_FP32) or doubles (MFEM_FP64). */
int mfem_batch_get_values(mfem_batch *batch, int item, int set, int precision, void *values);
int mfem_batch_get_prec(mfem_batch *batch, int item, int set, double *prec);
/* Items, elements over all items, element-assemblies per iteration (elements x
 * sets), work items and persistent grid size. */
int mfem_batch_info(mfem_batch *batch, int *nbItems, long long *nbElemTotal,
                    long long *nbAssemblies, int *nbWork, int *grid);

/* ---- self-test ------------------------------------------------------------- */
/* The FP64 kernels form part of their products on the integer pipes (a
 * correctly rounded multiplication with the FP64 unit's bits).  Compares that
 * multiplication with the FP64 unit on n seeded operand pairs on ctx's device:
 * *fastPath = pairs it handled, *mismatches = pairs whose bits differ (0). */
int mfem_selftest_dmul(mfem_context *ctx, long long n, unsigned long long seed,
                       unsigned long long *fastPath, unsigned long long *mismatches);
/* Measured FP64 pipe rate of ctx's device (no counterpart in the reference):
 * kind 0 = additions, 1 = fused multiply-adds, in operations per second (the
 * best of three timed launches of independent chains on every SM).  The FP64
 * gather's roofline is this pipe, not HBM. */
int mfem_fp64_rate(mfem_context *ctx, int kind, double *opsPerSecond);

/* ---- reference-shaped single calls (host buffers in and out) ---------------- */
/* Same arguments and meaning as the reference operators; each call uploads what
 * it reads and downloads what it writes.  nodeToNodeRow / nodeToNodeColumn must
 * describe the pattern (either the one mfem_create_nodeToNode returned, which is
 * recognised without re-upload, or any valid CSR of the mesh). */
int mfem_assembly(mfem_context *ctx, double *coord, double *nodeToNodeValue,
                  int *nodeToNodeRow, int *nodeToNodeColumn, int *elemToNode,
                  int *elemToEdge, int nbElem, int nbEdges, int operatorDim,
                  int operatorID);
int mfem_prec_init_host(mfem_context *ctx, double *prec, double *nodeToNodeValue,
                        int *nodeToNodeRow, int *nodeToNodeColumn, int nbNodes,
                        int operatorDim);
int mfem_prec_inversion_host(mfem_context *ctx, double *prec, int *nodeToNodeRow,
                             int *nodeToNodeColumn, int *checkBounds, int nbNodes,
                             int operatorID);

#ifdef __cplusplus
}
#endif
#endif
