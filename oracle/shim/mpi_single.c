/* Single-rank MPI calls for the oracle build of the reference sources.
 * A send to self is held until the matching receive is posted (or the
 * reverse), which is all that the reference's patch exchange does at
 * world size 1 (patches.c:242-315). */
#include <stdio.h>
#include <string.h>
#include <sys/types.h>
#include <unistd.h>
#include "mpi.h"

static size_t type_bytes(MPI_Datatype t)
{
    switch (t) {
    case MPI_INT: return sizeof(int);
    case MPI_BYTE: case MPI_CHAR: return 1;
    case MPI_DOUBLE: return sizeof(double);
    case MPI_DOUBLE_INT: return sizeof(double) + sizeof(int) + 4;
    case MPI_UINT64_T: case MPI_LONG_LONG: return 8;
    case MPI_FLOAT: return sizeof(float);
    default: return 1;
    }
}

int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
    (void)op; (void)c;
    if (s != MPI_IN_PLACE) memmove(r, s, (size_t)n * type_bytes(t));
    return MPI_SUCCESS;
}

int MPI_Alltoall(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c)
{
    (void)rn; (void)rt; (void)c;
    memmove(r, s, (size_t)sn * type_bytes(st));
    return MPI_SUCCESS;
}

int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c)
{
    return MPI_Alltoall(s, sn, st, r, rn, rt, c);
}

/* one pending message in each direction is enough for the reference's usage */
static const void *pend_send; static size_t pend_send_n;
static void *pend_recv; static size_t pend_recv_n;

int MPI_Isend(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c, MPI_Request *q)
{
    (void)dst; (void)tag; (void)c;
    size_t bytes = (size_t)n * type_bytes(t);
    if (pend_recv) {
        memcpy(pend_recv, b, bytes < pend_recv_n ? bytes : pend_recv_n);
        pend_recv = NULL;
    } else {
        pend_send = b; pend_send_n = bytes;
    }
    if (q) *q = 0;
    return MPI_SUCCESS;
}

int MPI_Irecv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Request *q)
{
    (void)src; (void)tag; (void)c;
    size_t bytes = (size_t)n * type_bytes(t);
    if (pend_send) {
        memcpy(b, pend_send, bytes < pend_send_n ? bytes : pend_send_n);
        pend_send = NULL;
    } else {
        pend_recv = b; pend_recv_n = bytes;
    }
    if (q) *q = 0;
    return MPI_SUCCESS;
}

int MPI_Wait(MPI_Request *q, MPI_Status *st) { (void)q; (void)st; return MPI_SUCCESS; }

int MPI_Abort(MPI_Comm c, int code)
{
    (void)c;
    fprintf(stderr, "MPI_Abort(%d) called by the reference oracle\n", code);
    exit(code);
}

int MPI_Get_processor_name(char *name, int *len)
{
    strcpy(name, "oracle");
    *len = 6;
    return MPI_SUCCESS;
}

int MPI_Cart_shift(MPI_Comm c, int dir, int disp, int *src, int *dst)
{
    (void)c; (void)dir; (void)disp;
    *src = MPI_PROC_NULL;
    *dst = MPI_PROC_NULL;
    return MPI_SUCCESS;
}

int MPI_File_open(MPI_Comm c, const char *name, int mode, MPI_Info info, MPI_File *fh)
{
    (void)c; (void)info;
    FILE *f = fopen(name, (mode & MPI_MODE_WRONLY) ? ((mode & MPI_MODE_CREATE) ? "w+b" : "r+b") : "rb");
    *fh = (MPI_File)f;
    return f ? MPI_SUCCESS : 1;
}

int MPI_File_set_size(MPI_File fh, MPI_Offset size)
{
    FILE *f = (FILE *)fh;
    if (!f) return 1;
    fflush(f);
    return ftruncate(fileno(f), (off_t)size) == 0 ? MPI_SUCCESS : 1;
}

int MPI_File_seek(MPI_File fh, MPI_Offset off, int whence)
{
    (void)whence;
    return fseeko((FILE *)fh, (off_t)off, SEEK_SET) == 0 ? MPI_SUCCESS : 1;
}

int MPI_File_write(MPI_File fh, const void *buf, int n, MPI_Datatype t, MPI_Status *st)
{
    (void)st;
    size_t bytes = (size_t)n * type_bytes(t);
    return fwrite(buf, 1, bytes, (FILE *)fh) == bytes ? MPI_SUCCESS : 1;
}

int MPI_File_close(MPI_File *fh)
{
    int rc = fclose((FILE *)*fh);
    *fh = NULL;
    return rc == 0 ? MPI_SUCCESS : 1;
}
