/* Test infrastructure: a single-process stand-in for the MPI library, enough
 * for the reference's host driver (src/axbc2d.c) and the MPI variant of its
 * Graph500 generator (generator/make_graph.c and friends) to compile unchanged
 * and run as one rank (-p 1x1).  Every communicator has one member (rank 0);
 * collectives copy the send buffer to the receive buffer; point-to-point
 * messages to oneself are matched against posted receives or queued; one-sided
 * gets read from the window's base.  Anything that would need a second rank
 * aborts with a message.  Built only by oracle/Makefile into oracle/_ref. */
#ifndef AXBC_REFHOST_MPI_H
#define AXBC_REFHOST_MPI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Win;
typedef ptrdiff_t MPI_Aint;
typedef struct {
    int MPI_SOURCE;
    int MPI_TAG;
    int MPI_ERROR;
    size_t bytes; /* payload received */
} MPI_Status;
typedef struct axbc_mpi_req *MPI_Request;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_COMM_NULL (-1)
#define MPI_INFO_NULL 0
#define MPI_REQUEST_NULL ((MPI_Request)0)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_MAX_PROCESSOR_NAME 256

/* datatypes: the handle indexes a size table (struct types are appended) */
#define MPI_DATATYPE_NULL 0
#define MPI_CHAR 1
#define MPI_UNSIGNED_CHAR 2
#define MPI_BYTE 3
#define MPI_INT 4
#define MPI_UNSIGNED 5
#define MPI_LONG 6
#define MPI_UNSIGNED_LONG 7
#define MPI_LONG_LONG 8
#define MPI_UNSIGNED_LONG_LONG 9
#define MPI_FLOAT 10
#define MPI_DOUBLE 11
#define MPI_UINT32_T 12
#define MPI_UINT64_T 13
#define MPI_INT64_T 14
#define MPI_INT32_T 15
#define MPI_SHORT 16
#define MPI_LONG_LONG_INT MPI_LONG_LONG

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_LOR 4
#define MPI_LAND 5
#define MPI_BOR 6
#define MPI_PROD 7

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm *out);
int MPI_Comm_free(MPI_Comm *comm);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Pcontrol(const int level, ...);
int MPI_Get_processor_name(char *name, int *len);

int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm);
int MPI_Allgather(const void *s, int scount, MPI_Datatype st, void *r, int rcount, MPI_Datatype rt,
                  MPI_Comm comm);
int MPI_Gather(const void *s, int scount, MPI_Datatype st, void *r, int rcount, MPI_Datatype rt,
               int root, MPI_Comm comm);
int MPI_Alltoall(const void *s, int scount, MPI_Datatype st, void *r, int rcount, MPI_Datatype rt,
                 MPI_Comm comm);
int MPI_Alltoallv(const void *s, const int *scounts, const int *sdispls, MPI_Datatype st, void *r,
                  const int *rcounts, const int *rdispls, MPI_Datatype rt, MPI_Comm comm);

int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Ssend(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Rsend(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Status *st);
int MPI_Irecv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Request *req);
int MPI_Isend(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Wait(MPI_Request *req, MPI_Status *st);
int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *sts);
int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *count);

int MPI_Get_address(const void *location, MPI_Aint *address);
int MPI_Type_struct(int count, const int *blocklens, const MPI_Aint *displs, const MPI_Datatype *types,
                    MPI_Datatype *out);
int MPI_Type_create_struct(int count, const int *blocklens, const MPI_Aint *displs,
                           const MPI_Datatype *types, MPI_Datatype *out);
int MPI_Type_commit(MPI_Datatype *t);
int MPI_Type_free(MPI_Datatype *t);

int MPI_Win_create(void *base, MPI_Aint size, int disp_unit, MPI_Info info, MPI_Comm comm, MPI_Win *win);
int MPI_Win_free(MPI_Win *win);
int MPI_Win_lock_all(int assert_, MPI_Win win);
int MPI_Win_unlock_all(MPI_Win win);
int MPI_Win_flush(int rank, MPI_Win win);
int MPI_Get(void *origin, int ocount, MPI_Datatype ot, int target, MPI_Aint tdisp, int tcount,
            MPI_Datatype tt, MPI_Win win);

#ifdef __cplusplus
}
#endif
#endif
