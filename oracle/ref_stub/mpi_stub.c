/* One-rank definitions of the MPI calls declared in ref_stub/mpi.h (test infrastructure:
 * links the reference's CPU sources into oracle/_ref without an MPI installation). */
#include "mpi.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
static size_t tsize(MPI_Datatype t) { return t == MPI_DOUBLE ? sizeof(double) : sizeof(int); }
int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Abort(MPI_Comm c, int code) { (void)c; exit(code); }
int MPI_Comm_size(MPI_Comm c, int *size) { (void)c; *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm c, int *rank) { (void)c; *rank = 0; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
int MPI_Error_string(int code, char *s, int *len) { *len = snprintf(s, MPI_MAX_ERROR_STRING, "mpi stub error %d", code); return 0; }
int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int g, MPI_Comm c) { (void)b; (void)n; (void)t; (void)d; (void)g; (void)c; fprintf(stderr, "mpi stub: Send on one rank\n"); exit(3); }
int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int g, MPI_Comm c, MPI_Status *st) { (void)b; (void)n; (void)t; (void)s; (void)g; (void)c; (void)st; fprintf(stderr, "mpi stub: Recv on one rank\n"); exit(3); }
int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int g, MPI_Comm c, MPI_Request *r) { (void)b; (void)n; (void)t; (void)d; (void)g; (void)c; (void)r; fprintf(stderr, "mpi stub: Isend on one rank\n"); exit(3); }
int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int g, MPI_Comm c, MPI_Request *r) { (void)b; (void)n; (void)t; (void)s; (void)g; (void)c; (void)r; fprintf(stderr, "mpi stub: Irecv on one rank\n"); exit(3); }
int MPI_Waitall(int n, MPI_Request *r, MPI_Status *st) { (void)n; (void)r; (void)st; return 0; }
int MPI_Waitany(int n, MPI_Request *r, int *idx, MPI_Status *st) { (void)n; (void)r; (void)st; *idx = -1; return 0; }
int MPI_Request_free(MPI_Request *r) { (void)r; return 0; }
int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c) { (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c) { (void)op; (void)c; memmove(r, s, tsize(t) * (size_t)n); return 0; }
int MPI_Scatter(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int root, MPI_Comm c) { (void)sn; (void)root; (void)c; (void)st; memmove(r, s, tsize(rt) * (size_t)rn); return 0; }
int MPI_Scatterv(const void *s, const int *sc, const int *dis, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int root, MPI_Comm c) { (void)sc; (void)root; (void)c; memmove(r, (const char *)s + tsize(st) * (size_t)dis[0], tsize(rt) * (size_t)rn); return 0; }
int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int root, MPI_Comm c) { (void)rn; (void)rt; (void)root; (void)c; memmove(r, s, tsize(st) * (size_t)sn); return 0; }
int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *rc, const int *dis, MPI_Datatype rt, int root, MPI_Comm c) { (void)rc; (void)rt; (void)root; (void)c; memmove((char *)r + tsize(st) * (size_t)dis[0], s, tsize(st) * (size_t)sn); return 0; }
