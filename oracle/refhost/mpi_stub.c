/* Test infrastructure: the single-process MPI stand-in declared in mpi.h.
 * One rank everywhere; see mpi.h for what each call does. */
#include "mpi.h"

#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static void die(const char *what)
{
    fprintf(stderr, "single-rank MPI stand-in: %s needs more than one rank\n", what);
    exit(3);
}

/* ------------------------------------------------------------ datatypes */
#define MAX_TYPES 64
static size_t type_size[MAX_TYPES] = {
    0, /* NULL */ 1, 1, 1, 4, 4, sizeof(long), sizeof(unsigned long), 8, 8, 4, 8, 4, 8, 8, 4, 2};
static int n_types = 17;

static size_t tsize(MPI_Datatype t)
{
    if (t < 0 || t >= n_types) die("an unknown datatype");
    return type_size[t];
}

int MPI_Get_address(const void *location, MPI_Aint *address)
{
    *address = (MPI_Aint)(uintptr_t)location;
    return MPI_SUCCESS;
}

int MPI_Type_struct(int count, const int *blocklens, const MPI_Aint *displs, const MPI_Datatype *types,
                    MPI_Datatype *out)
{
    /* extent = end of the last member relative to the first displacement,
     * rounded up to the largest member alignment (8 for the types used) */
    MPI_Aint lo = displs[0], hi = displs[0];
    size_t align = 1;
    for (int i = 0; i < count; i++) {
        const MPI_Aint end = displs[i] + (MPI_Aint)(blocklens[i] * tsize(types[i]));
        if (displs[i] < lo) lo = displs[i];
        if (end > hi) hi = end;
        if (tsize(types[i]) > align) align = tsize(types[i]);
    }
    size_t ext = (size_t)(hi - lo);
    ext = (ext + align - 1) / align * align;
    if (n_types >= MAX_TYPES) die("too many derived datatypes");
    type_size[n_types] = ext;
    *out = n_types++;
    return MPI_SUCCESS;
}

int MPI_Type_create_struct(int count, const int *blocklens, const MPI_Aint *displs,
                           const MPI_Datatype *types, MPI_Datatype *out)
{
    return MPI_Type_struct(count, blocklens, displs, types, out);
}

int MPI_Type_commit(MPI_Datatype *t)
{
    (void)t;
    return MPI_SUCCESS;
}

int MPI_Type_free(MPI_Datatype *t)
{
    *t = MPI_DATATYPE_NULL;
    return MPI_SUCCESS;
}

/* ------------------------------------------------------------ environment */
int MPI_Init(int *argc, char ***argv)
{
    (void)argc;
    (void)argv;
    return MPI_SUCCESS;
}

int MPI_Finalize(void) { return MPI_SUCCESS; }

int MPI_Abort(MPI_Comm comm, int code)
{
    (void)comm;
    fprintf(stderr, "MPI_Abort(%d)\n", code);
    exit(code ? code : 1);
}

int MPI_Comm_rank(MPI_Comm comm, int *rank)
{
    (void)comm;
    *rank = 0;
    return MPI_SUCCESS;
}

int MPI_Comm_size(MPI_Comm comm, int *size)
{
    (void)comm;
    *size = 1;
    return MPI_SUCCESS;
}

static int next_comm = 1;
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm *out)
{
    (void)comm;
    (void)color;
    (void)key;
    *out = next_comm++;
    return MPI_SUCCESS;
}

int MPI_Comm_free(MPI_Comm *comm)
{
    *comm = MPI_COMM_NULL;
    return MPI_SUCCESS;
}

int MPI_Barrier(MPI_Comm comm)
{
    (void)comm;
    return MPI_SUCCESS;
}

double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int MPI_Pcontrol(const int level, ...)
{
    (void)level;
    return MPI_SUCCESS;
}

int MPI_Get_processor_name(char *name, int *len)
{
    strcpy(name, "localhost");
    *len = 9;
    return MPI_SUCCESS;
}

/* ------------------------------------------------------------ collectives */
static void copy_if(const void *s, void *r, size_t bytes)
{
    if (s == MPI_IN_PLACE || r == NULL || s == r || bytes == 0) return;
    memmove(r, s, bytes);
}

int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm)
{
    (void)buf;
    (void)count;
    (void)t;
    (void)comm;
    if (root != 0) die("MPI_Bcast from a root other than 0");
    return MPI_SUCCESS;
}

int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, MPI_Comm comm)
{
    (void)op;
    (void)comm;
    copy_if(s, r, (size_t)count * tsize(t));
    return MPI_SUCCESS;
}

int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm comm)
{
    (void)op;
    (void)comm;
    if (root != 0) die("MPI_Reduce to a root other than 0");
    copy_if(s, r, (size_t)count * tsize(t));
    return MPI_SUCCESS;
}

int MPI_Allgather(const void *s, int scount, MPI_Datatype st, void *r, int rcount, MPI_Datatype rt,
                  MPI_Comm comm)
{
    (void)rcount;
    (void)rt;
    (void)comm;
    copy_if(s, r, (size_t)scount * tsize(st));
    return MPI_SUCCESS;
}

int MPI_Gather(const void *s, int scount, MPI_Datatype st, void *r, int rcount, MPI_Datatype rt,
               int root, MPI_Comm comm)
{
    (void)rcount;
    (void)rt;
    (void)comm;
    if (root != 0) die("MPI_Gather to a root other than 0");
    copy_if(s, r, (size_t)scount * tsize(st));
    return MPI_SUCCESS;
}

int MPI_Alltoall(const void *s, int scount, MPI_Datatype st, void *r, int rcount, MPI_Datatype rt,
                 MPI_Comm comm)
{
    (void)rcount;
    (void)rt;
    (void)comm;
    copy_if(s, r, (size_t)scount * tsize(st));
    return MPI_SUCCESS;
}

int MPI_Alltoallv(const void *s, const int *scounts, const int *sdispls, MPI_Datatype st, void *r,
                  const int *rcounts, const int *rdispls, MPI_Datatype rt, MPI_Comm comm)
{
    (void)rcounts;
    (void)comm;
    if (s == MPI_IN_PLACE) return MPI_SUCCESS;
    memmove((char *)r + (size_t)rdispls[0] * tsize(rt), (const char *)s + (size_t)sdispls[0] * tsize(st),
            (size_t)scounts[0] * tsize(st));
    return MPI_SUCCESS;
}

/* ------------------------------------------------------------ point to point
 * Messages to oneself: a send completes a matching posted receive, or is
 * queued until one is posted. */
struct axbc_mpi_req {
    void *buf;
    size_t cap;
    int tag;
    int done;
    size_t bytes;
    struct axbc_mpi_req *next;
};
struct queued_msg {
    int tag;
    size_t bytes;
    void *data;
    struct queued_msg *next;
};
static struct axbc_mpi_req *posted = NULL;
static struct queued_msg *queued = NULL;

static void self_only(int peer, const char *what)
{
    if (peer != 0 && peer != MPI_ANY_SOURCE) die(what);
}

static int tag_match(int want, int got) { return want == MPI_ANY_TAG || want == got; }

static int deliver(const void *buf, size_t bytes, int tag)
{
    struct axbc_mpi_req **pp = &posted;
    for (; *pp; pp = &(*pp)->next) {
        struct axbc_mpi_req *q = *pp;
        if (!tag_match(q->tag, tag)) continue;
        if (bytes > q->cap) die("a message longer than its receive buffer");
        memcpy(q->buf, buf, bytes);
        q->bytes = bytes;
        q->done = 1;
        *pp = q->next;
        return 1;
    }
    struct queued_msg *m = (struct queued_msg *)malloc(sizeof(*m));
    m->tag = tag;
    m->bytes = bytes;
    m->data = malloc(bytes ? bytes : 1);
    memcpy(m->data, buf, bytes);
    m->next = NULL;
    struct queued_msg **tail = &queued;
    while (*tail) tail = &(*tail)->next;
    *tail = m;
    return 0;
}

static int take_queued(struct axbc_mpi_req *q)
{
    struct queued_msg **pp = &queued;
    for (; *pp; pp = &(*pp)->next) {
        struct queued_msg *m = *pp;
        if (!tag_match(q->tag, m->tag)) continue;
        if (m->bytes > q->cap) die("a message longer than its receive buffer");
        memcpy(q->buf, m->data, m->bytes);
        q->bytes = m->bytes;
        q->done = 1;
        *pp = m->next;
        free(m->data);
        free(m);
        return 1;
    }
    return 0;
}

static int send_self(const void *buf, int count, MPI_Datatype t, int dest, int tag)
{
    self_only(dest, "a send to another rank");
    deliver(buf, (size_t)count * tsize(t), tag);
    return MPI_SUCCESS;
}

int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm)
{
    (void)comm;
    return send_self(buf, count, t, dest, tag);
}

int MPI_Ssend(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm)
{
    (void)comm;
    return send_self(buf, count, t, dest, tag);
}

int MPI_Rsend(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm)
{
    (void)comm;
    return send_self(buf, count, t, dest, tag);
}

int MPI_Isend(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm comm,
              MPI_Request *req)
{
    (void)comm;
    send_self(buf, count, t, dest, tag);
    *req = MPI_REQUEST_NULL;
    return MPI_SUCCESS;
}

int MPI_Irecv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Request *req)
{
    (void)comm;
    self_only(src, "a receive from another rank");
    struct axbc_mpi_req *q = (struct axbc_mpi_req *)calloc(1, sizeof(*q));
    q->buf = buf;
    q->cap = (size_t)count * tsize(t);
    q->tag = tag;
    if (!take_queued(q)) {
        struct axbc_mpi_req **tail = &posted;
        while (*tail) tail = &(*tail)->next;
        *tail = q;
    }
    *req = q;
    return MPI_SUCCESS;
}

int MPI_Wait(MPI_Request *req, MPI_Status *st)
{
    struct axbc_mpi_req *q = *req;
    if (!q) return MPI_SUCCESS;
    if (!q->done && !take_queued(q)) die("a receive that no send on this rank completes");
    if (st) {
        st->MPI_SOURCE = 0;
        st->MPI_TAG = q->tag;
        st->MPI_ERROR = 0;
        st->bytes = q->bytes;
    }
    free(q);
    *req = MPI_REQUEST_NULL;
    return MPI_SUCCESS;
}

int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *sts)
{
    for (int i = 0; i < n; i++) MPI_Wait(&reqs[i], sts ? &sts[i] : NULL);
    return MPI_SUCCESS;
}

int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm comm, MPI_Status *st)
{
    MPI_Request r;
    MPI_Irecv(buf, count, t, src, tag, comm, &r);
    return MPI_Wait(&r, st);
}

int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *count)
{
    *count = (int)(st->bytes / tsize(t));
    return MPI_SUCCESS;
}

/* ------------------------------------------------------------ one-sided */
#define MAX_WINS 16
static struct {
    char *base;
    int unit;
    int used;
} wins[MAX_WINS];

int MPI_Win_create(void *base, MPI_Aint size, int disp_unit, MPI_Info info, MPI_Comm comm, MPI_Win *win)
{
    (void)size;
    (void)info;
    (void)comm;
    for (int i = 0; i < MAX_WINS; i++)
        if (!wins[i].used) {
            wins[i].base = (char *)base;
            wins[i].unit = disp_unit;
            wins[i].used = 1;
            *win = i;
            return MPI_SUCCESS;
        }
    die("more windows than the stand-in holds");
    return 1;
}

int MPI_Win_free(MPI_Win *win)
{
    wins[*win].used = 0;
    *win = -1;
    return MPI_SUCCESS;
}

int MPI_Win_lock_all(int assert_, MPI_Win win)
{
    (void)assert_;
    (void)win;
    return MPI_SUCCESS;
}

int MPI_Win_unlock_all(MPI_Win win)
{
    (void)win;
    return MPI_SUCCESS;
}

int MPI_Win_flush(int rank, MPI_Win win)
{
    (void)rank;
    (void)win;
    return MPI_SUCCESS;
}

int MPI_Get(void *origin, int ocount, MPI_Datatype ot, int target, MPI_Aint tdisp, int tcount,
            MPI_Datatype tt, MPI_Win win)
{
    (void)tcount;
    (void)tt;
    self_only(target, "a one-sided get from another rank");
    memcpy(origin, wins[win].base + (size_t)tdisp * (size_t)wins[win].unit, (size_t)ocount * tsize(ot));
    return MPI_SUCCESS;
}
