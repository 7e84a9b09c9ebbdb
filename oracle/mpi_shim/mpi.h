/*
 * Single-rank MPI stand-in used only to compile the reference C sources of
 * MetaPart (genHistograms.c, metapart.c) into the CPU checker under
 * oracle/_ref/.  It is test infrastructure: nothing in the GPU product links it.
 *
 * Semantics implemented (one process, rank 0, world size 1):
 *   - MPI_File_* map to POSIX open/pread/pwrite (MPI_MODE_CREATE does not
 *     truncate, as in MPI-IO); MPI_Get_count returns the bytes moved.
 *   - Reductions with MPI_IN_PLACE are identities; with distinct buffers they
 *     copy.  Alltoall / Bcast / Barrier are copies or no-ops.
 *   - Point-to-point calls are never reached at one rank (the reference only
 *     issues them when numTasks > 1); they abort if called.
 */
#ifndef MP_MPI_SHIM_H
#define MP_MPI_SHIM_H

#include <fcntl.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>
#include <sys/types.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Request;
typedef long long MPI_Offset;
typedef struct { int fd; } mp_shim_file;
typedef mp_shim_file *MPI_File;
typedef struct { long long count; int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_THREAD_MULTIPLE 3
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1
#define MPI_IN_PLACE ((void *)1)

enum { MPI_BYTE = 1, MPI_INT, MPI_UNSIGNED, MPI_UNSIGNED_LONG, MPI_UNSIGNED_SHORT };
enum { MPI_SUM = 1, MPI_MAX, MPI_BOR };

static inline size_t mp_shim_tsize(MPI_Datatype t)
{
    switch (t) {
    case MPI_BYTE: return 1;
    case MPI_INT: return sizeof(int);
    case MPI_UNSIGNED: return sizeof(unsigned);
    case MPI_UNSIGNED_LONG: return sizeof(unsigned long);
    case MPI_UNSIGNED_SHORT: return sizeof(unsigned short);
    default: return 1;
    }
}

static inline void mp_shim_unreachable(const char *what)
{
    fprintf(stderr, "mpi shim: %s is not available at one rank\n", what);
    abort();
}

static inline int MPI_Init_thread(int *argc, char ***argv, int req, int *prov)
{ (void)argc; (void)argv; *prov = req; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *n) { (void)c; *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Type_size(MPI_Datatype t, int *s) { *s = (int)mp_shim_tsize(t); return 0; }

static inline int MPI_File_open(MPI_Comm c, const char *name, int mode, MPI_Info info, MPI_File *fh)
{
    (void)c; (void)info;
    int flags = (mode & MPI_MODE_WRONLY) ? O_WRONLY : O_RDONLY;
    if (mode & MPI_MODE_CREATE) flags |= O_CREAT;
    int fd = open(name, flags, 0644);
    if (fd < 0) { *fh = NULL; return 1; }
    *fh = (MPI_File)malloc(sizeof(mp_shim_file));
    (*fh)->fd = fd;
    return 0;
}
static inline int MPI_File_close(MPI_File *fh)
{
    if (*fh) { close((*fh)->fd); free(*fh); *fh = NULL; }
    return 0;
}
static inline int MPI_File_read_at(MPI_File fh, MPI_Offset off, void *buf, long long count,
                                   MPI_Datatype t, MPI_Status *st)
{
    size_t want = (size_t)count * mp_shim_tsize(t), got = 0;
    while (got < want) {
        ssize_t r = pread(fh->fd, (char *)buf + got, want - got, (off_t)off + (off_t)got);
        if (r <= 0) break;
        got += (size_t)r;
    }
    if (st) st->count = (long long)got;
    return 0;
}
static inline int MPI_File_write_at(MPI_File fh, MPI_Offset off, const void *buf, long long count,
                                    MPI_Datatype t, MPI_Status *st)
{
    size_t want = (size_t)count * mp_shim_tsize(t), put = 0;
    while (put < want) {
        ssize_t r = pwrite(fh->fd, (const char *)buf + put, want - put, (off_t)off + (off_t)put);
        if (r <= 0) break;
        put += (size_t)r;
    }
    if (st) st->count = (long long)put;
    return 0;
}
static inline int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *count)
{ *count = (int)(st->count / (long long)mp_shim_tsize(t)); return 0; }

static inline int MPI_Allreduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
    (void)op; (void)c;
    if (sb != MPI_IN_PLACE && sb != rb) memcpy(rb, sb, (size_t)n * mp_shim_tsize(t));
    return 0;
}
static inline int MPI_Reduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c)
{
    (void)root;
    return MPI_Allreduce(sb, rb, n, t, op, c);
}
static inline int MPI_Alltoall(const void *sb, int sn, MPI_Datatype st, void *rb, int rn,
                               MPI_Datatype rt, MPI_Comm c)
{
    (void)rn; (void)rt; (void)c;
    if (sb != rb) memcpy(rb, sb, (size_t)sn * mp_shim_tsize(st));
    return 0;
}
static inline int MPI_Bcast(void *b, int n, MPI_Datatype t, int root, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)root; (void)c; return 0; }

static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; mp_shim_unreachable("MPI_Send"); return 1; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; mp_shim_unreachable("MPI_Recv"); return 1; }
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *r)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; (void)r; mp_shim_unreachable("MPI_Isend"); return 1; }
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *r)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)r; mp_shim_unreachable("MPI_Irecv"); return 1; }
static inline int MPI_Waitall(int n, MPI_Request *r, MPI_Status *st)
{ (void)r; (void)st; if (n > 0) mp_shim_unreachable("MPI_Waitall"); return 0; }
static inline int MPI_Iprobe(int s, int tag, MPI_Comm c, int *flag, MPI_Status *st)
{ (void)s; (void)tag; (void)c; (void)st; *flag = 0; return 0; }
static inline int MPI_Gather(const void *sb, int sn, MPI_Datatype st, void *rb, int rn, MPI_Datatype rt,
                             int root, MPI_Comm c)
{ (void)rn; (void)rt; (void)root; (void)c; if (sb != rb) memcpy(rb, sb, (size_t)sn * mp_shim_tsize(st)); return 0; }
static inline int MPI_Gatherv(const void *sb, int sn, MPI_Datatype st, void *rb, const int *rc,
                              const int *disp, MPI_Datatype rt, int root, MPI_Comm c)
{
    (void)rc; (void)rt; (void)root; (void)c;
    memcpy((char *)rb + (size_t)disp[0] * mp_shim_tsize(st), sb, (size_t)sn * mp_shim_tsize(st));
    return 0;
}

#endif
