/* Oracle (test infrastructure only): single-rank stand-in for <mpi.h>.
 * The reference's REF build runs with one rank here: MPI_Comm_size reports 1,
 * so the halo exchange (src/halo.cc:44) and the timer reduction
 * (src/FEM.cc:111) are never entered; their calls still have to compile. */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int dummy; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_UINT64_T 2
#define MPI_INT 3
#define MPI_MAX 0
#define MPI_SUM 1
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

static inline int MPI_Init (int *, char ***) { return 0; }
static inline int MPI_Finalize () { return 0; }
static inline int MPI_Comm_size (MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Comm_rank (MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Irecv (void *, int, MPI_Datatype, int, int, MPI_Comm,
                             MPI_Request *) { return 0; }
static inline int MPI_Send (const void *, int, MPI_Datatype, int, int, MPI_Comm)
{ return 0; }
static inline int MPI_Waitall (int, MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Reduce (const void *, void *, int, MPI_Datatype, MPI_Op, int,
                              MPI_Comm) { return 0; }
#endif
