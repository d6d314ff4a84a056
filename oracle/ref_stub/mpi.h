/* Single-rank stand-in for <mpi.h>, used only to compile the reference's CPU sources into
 * oracle/_ref (the machines here have no MPI). Only the names those sources mention exist;
 * every call behaves as on a one-rank MPI_COMM_WORLD. Test infrastructure, not product code. */
#ifndef HHP_REF_STUB_MPI_H
#define HHP_REF_STUB_MPI_H
#include <stddef.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_SUM 1
#define MPI_SUCCESS 0
#define MPI_MAX_ERROR_STRING 64
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm c, int code);
int MPI_Comm_size(MPI_Comm c, int *size);
int MPI_Comm_rank(MPI_Comm c, int *rank);
int MPI_Barrier(MPI_Comm c);
int MPI_Error_string(int code, char *s, int *len);
int MPI_Send(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c);
int MPI_Recv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *st);
int MPI_Isend(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c, MPI_Request *r);
int MPI_Irecv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Request *r);
int MPI_Waitall(int n, MPI_Request *r, MPI_Status *st);
int MPI_Waitany(int n, MPI_Request *r, int *idx, MPI_Status *st);
int MPI_Request_free(MPI_Request *r);
int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c);
int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Scatter(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int root, MPI_Comm c);
int MPI_Scatterv(const void *s, const int *sc, const int *dis, MPI_Datatype st, void *r, int rn, MPI_Datatype rt,
                 int root, MPI_Comm c);
int MPI_Gather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, int root, MPI_Comm c);
int MPI_Gatherv(const void *s, int sn, MPI_Datatype st, void *r, const int *rc, const int *dis, MPI_Datatype rt,
                int root, MPI_Comm c);
#endif
