/* Single-rank stand-in for <mpi.h>, used only to compile the reference's
 * hot-path sources into the test oracle library (oracle/_ref).  Every
 * collective and point-to-point call acts on a world of exactly one rank.
 * Test infrastructure: nothing in the product links against this. */
#ifndef TM_SHIM_MPI_H
#define TM_SHIM_MPI_H
#include <stdint.h>
#include <stdlib.h>
#include <limits.h>

typedef int MPI_Comm;
typedef int MPI_Request;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_INT 1
#define MPI_BYTE 2
#define MPI_DOUBLE 3
#define MPI_DOUBLE_INT 4
#define MPI_UINT64_T 5
#define MPI_LONG_LONG 6
#define MPI_CHAR 7
#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3
#define MPI_MINLOC 4
#define MPI_IN_PLACE ((void *)1)
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_PROC_NULL (-2)
#define MPI_FLOAT 8
#define MPI_INFO_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1
#define MPI_MODE_RDONLY 2
#define MPI_SEEK_SET 600
typedef long long MPI_Offset;
typedef void *MPI_File;   /* a stdio FILE at one rank */
typedef int MPI_Info;

int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Alltoall(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c);
int MPI_Allgather(const void *s, int sn, MPI_Datatype st, void *r, int rn, MPI_Datatype rt, MPI_Comm c);
int MPI_Isend(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c, MPI_Request *q);
int MPI_Irecv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Request *q);
int MPI_Wait(MPI_Request *q, MPI_Status *st);
int MPI_Abort(MPI_Comm c, int code);
int MPI_Get_processor_name(char *name, int *len);
/* MPI-IO at one rank: a plain file */
int MPI_File_open(MPI_Comm c, const char *name, int mode, MPI_Info info, MPI_File *fh);
int MPI_File_set_size(MPI_File fh, MPI_Offset size);
int MPI_File_seek(MPI_File fh, MPI_Offset off, int whence);
int MPI_File_write(MPI_File fh, const void *buf, int n, MPI_Datatype t, MPI_Status *st);
int MPI_File_close(MPI_File *fh);
/* one rank on a non-periodic grid: every neighbour is MPI_PROC_NULL */
int MPI_Cart_shift(MPI_Comm c, int dir, int disp, int *src, int *dst);
#endif
