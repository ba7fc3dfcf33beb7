/* Single-rank MPI stand-in for the oracle build (see mpi.h). */
#include "mpi.h"
#include <string.h>
#include <time.h>

int MPI_Init(int* argc, char*** argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm c, int* r) { (void)c; *r = 0; return 0; }
int MPI_Comm_size(MPI_Comm c, int* s) { (void)c; *s = 1; return 0; }
int MPI_Comm_dup(MPI_Comm c, MPI_Comm* o) { *o = c; return 0; }
int MPI_Comm_free(MPI_Comm* c) { *c = MPI_COMM_NULL; return 0; }
int MPI_Comm_split(MPI_Comm c, int color, int key, MPI_Comm* o) { (void)key; *o = (color == MPI_UNDEFINED) ? MPI_COMM_NULL : c; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
double MPI_Wtime(void) { struct timespec t; clock_gettime(CLOCK_MONOTONIC, &t); return t.tv_sec + 1e-9 * t.tv_nsec; }
int MPI_Bcast(void* b, int n, MPI_Datatype t, int root, MPI_Comm c) { (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }

static void cp(const void* s, void* r, long bytes) { if (s != r && bytes > 0) memmove(r, s, (size_t)bytes); }

int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) { (void)op; (void)c; cp(s, r, (long)n * t); return 0; }
int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c) { (void)op; (void)root; (void)c; if (r) cp(s, r, (long)n * t); return 0; }
int MPI_Scan(const void* s, void* r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) { (void)op; (void)c; cp(s, r, (long)n * t); return 0; }
int MPI_Allgather(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, MPI_Comm c) { (void)rc; (void)rt; (void)c; cp(s, r, (long)sc * st); return 0; }
int MPI_Gather(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, int root, MPI_Comm c) { (void)rc; (void)rt; (void)root; (void)c; if (r) cp(s, r, (long)sc * st); return 0; }
int MPI_Gatherv(const void* s, int sc, MPI_Datatype st, void* r, const int* rcs, const int* d, MPI_Datatype rt, int root, MPI_Comm c)
{ (void)rcs; (void)root; (void)c; if (r) cp(s, (char*)r + (long)(d ? d[0] : 0) * rt, (long)sc * st); return 0; }
int MPI_Scatter(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, int root, MPI_Comm c) { (void)sc; (void)st; (void)root; (void)c; if (s) cp(s, r, (long)rc * rt); return 0; }
int MPI_Scatterv(const void* s, const int* scs, const int* d, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, int root, MPI_Comm c)
{ (void)scs; (void)root; (void)c; if (s) cp((const char*)s + (long)(d ? d[0] : 0) * st, r, (long)rc * rt); return 0; }
int MPI_Alltoall(const void* s, int sc, MPI_Datatype st, void* r, int rc, MPI_Datatype rt, MPI_Comm c) { (void)rc; (void)rt; (void)c; cp(s, r, (long)sc * st); return 0; }
int MPI_Send(const void* b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c) { (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return 0; }
int MPI_Recv(void* b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status* st) { (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; return 0; }
int MPI_Isend(const void* b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request* q) { (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; if (q) *q = 0; return 0; }
int MPI_Irecv(void* b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request* q) { (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; if (q) *q = 0; return 0; }
int MPI_Wait(MPI_Request* q, MPI_Status* st) { (void)q; (void)st; return 0; }
int MPI_Waitall(int n, MPI_Request* q, MPI_Status* st) { (void)n; (void)q; (void)st; return 0; }
int MPI_Test(MPI_Request* q, int* f, MPI_Status* st) { (void)q; (void)st; *f = 1; return 0; }

/* Graph partitioning is never reached with a single rank; fail loudly if it is. */
#include "parmetis.h"
#include <stdio.h>
#include <stdlib.h>
static int no_partitioner(void) { fprintf(stderr, "graph partitioner called in single-rank oracle build\n"); abort(); return METIS_ERROR; }
int ParMETIS_V3_PartKway(idx_t* a, idx_t* b, idx_t* c, idx_t* d, idx_t* e, idx_t* f, idx_t* g, idx_t* h, idx_t* i,
                         real_t* j, real_t* k, idx_t* l, idx_t* m, idx_t* n, MPI_Comm* o)
{ (void)a;(void)b;(void)c;(void)d;(void)e;(void)f;(void)g;(void)h;(void)i;(void)j;(void)k;(void)l;(void)m;(void)n;(void)o; return no_partitioner(); }
int METIS_PartGraphKway(idx_t* a, idx_t* b, idx_t* c, idx_t* d, idx_t* e, idx_t* f, idx_t* g, idx_t* h, real_t* i,
                        real_t* j, idx_t* k, idx_t* l, idx_t* m)
{ (void)a;(void)b;(void)c;(void)d;(void)e;(void)f;(void)g;(void)h;(void)i;(void)j;(void)k;(void)l;(void)m; return no_partitioner(); }
int METIS_PartGraphRecursive(idx_t* a, idx_t* b, idx_t* c, idx_t* d, idx_t* e, idx_t* f, idx_t* g, idx_t* h, real_t* i,
                             real_t* j, idx_t* k, idx_t* l, idx_t* m)
{ (void)a;(void)b;(void)c;(void)d;(void)e;(void)f;(void)g;(void)h;(void)i;(void)j;(void)k;(void)l;(void)m; return no_partitioner(); }
