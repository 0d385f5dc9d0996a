/*
 * Single-rank MPI shim used ONLY to compile the reference solver's own
 * sources (src/WENOFD.cpp of infinity-07/FD-WENO-EulerEquation) on a machine
 * without an MPI installation.  It is test infrastructure for the oracle, not
 * part of the product.
 *
 * Semantics: one process, rank 0 of size 1.  Collectives copy the send buffer
 * to the receive buffer.  Point-to-point messages go to the same process and
 * are matched by tag, which is what the reference's periodic halo exchange
 * with itself needs (src/WENOFD.cpp:897-902 posts Irecv with tags 1/2 and then
 * Isends with the same tags to itself).  MPI_Abort throws
 * std::runtime_error so the driver can report the failure instead of the
 * process dying.  MPI-IO maps onto stdio.
 */
#ifndef WENOFD_ORACLE_MPI_SHIM_H
#define WENOFD_ORACLE_MPI_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef struct MPI_Status { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
typedef struct wenofd_shim_file *MPI_File;

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_SUCCESS 0

#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_CHAR 3
#define MPI_OFFSET 4

#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_SUM 3

#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 4

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
double MPI_Wtime(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Barrier(MPI_Comm comm);

int MPI_Allgather(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf, int rcount,
                  MPI_Datatype rtype, MPI_Comm comm);
int MPI_Reduce(const void *sbuf, void *rbuf, int count, MPI_Datatype type, MPI_Op op, int root,
               MPI_Comm comm);
int MPI_Allreduce(const void *sbuf, void *rbuf, int count, MPI_Datatype type, MPI_Op op,
                  MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Exscan(const void *sbuf, void *rbuf, int count, MPI_Datatype type, MPI_Op op,
               MPI_Comm comm);

int MPI_Irecv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dst, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Waitall(int count, MPI_Request *reqs, MPI_Status *statuses);
int MPI_Recv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm,
             MPI_Status *status);
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dst, int tag, MPI_Comm comm);

int MPI_File_open(MPI_Comm comm, const char *name, int amode, MPI_Info info, MPI_File *fh);
int MPI_File_set_size(MPI_File fh, MPI_Offset size);
int MPI_File_write_at(MPI_File fh, MPI_Offset offset, const void *buf, int count,
                      MPI_Datatype type, MPI_Status *status);
int MPI_File_close(MPI_File *fh);

#ifdef __cplusplus
}
#endif

#endif
