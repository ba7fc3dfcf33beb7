/* Single-rank MPI stand-in used only to compile the reference simulator as a
 * test oracle on a host without an MPI library.  Every communicator has one
 * rank (rank 0); collectives copy the send buffer into the receive buffer and
 * point-to-point calls never happen because a single rank owns no ghost cells.
 * This is harness code for the oracle build, not part of the product. */
#ifndef OCPX_ORACLE_MPI_STUB_H
#define OCPX_ORACLE_MPI_STUB_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_COMM_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_SUCCESS 0
#define MPI_UNDEFINED (-32766)

/* datatype handle = element size in bytes */
#define MPI_CHAR 1
#define MPI_BYTE 1
#define MPI_INT 4
#define MPI_UNSIGNED 4
#define MPI_LONG 8
#define MPI_LONG_LONG_INT 8
#define MPI_UNSIGNED_LONG_LONG 8
#define MPI_DOUBLE 8
#define MPI_LONG_DOUBLE 16

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_LAND 4

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm* out);
int MPI_Comm_free(MPI_Comm* comm);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* out);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Bcast(void* buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Allreduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
int MPI_Scan(const void* s, void* r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Allgather(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, MPI_Comm comm);
int MPI_Gather(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Gatherv(const void* s, int sc, MPI_Datatype st, void* r, const int* rcs, const int* displs,
                MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Scatter(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Scatterv(const void* s, const int* scs, const int* displs, MPI_Datatype st, void* r, int rc,
                 MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Alltoall(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, MPI_Comm comm);
int MPI_Send(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Status* st);
int MPI_Isend(const void* buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm, MPI_Request* rq);
int MPI_Irecv(void* buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Request* rq);
int MPI_Wait(MPI_Request* rq, MPI_Status* st);
int MPI_Waitall(int n, MPI_Request* rq, MPI_Status* st);
int MPI_Test(MPI_Request* rq, int* flag, MPI_Status* st);

#ifdef __cplusplus
}
#endif
#endif
