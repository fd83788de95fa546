/*
 * Single-rank stand-in for the MPI interface that RNNG's headers and drivers use.
 *
 * The GB300 build runs the whole epsilon-graph / Rips pipeline on one GPU in one
 * process, so every communicator has exactly one rank (rank 0, size 1).  This
 * header declares the subset of MPI-3 that RNNG calls (include/point.hpp,
 * include/graph.hpp, include/simplex.hpp and the three drivers) with P = 1 semantics:
 *
 *   - collectives copy the send buffer to the receive buffer (MPI_IN_PLACE: no-op);
 *   - MPI_Exscan leaves the receive buffer untouched (undefined on rank 0 in MPI);
 *   - point-to-point messages to self are matched by tag and copied at post time;
 *   - MPI-IO maps onto POSIX pread/pwrite, honouring the file view's
 *     displacement and the resized extent of the file type.
 *
 * No network library is linked.  Where a real MPI is installed, build against
 * that instead; nothing in the GPU library depends on this file.
 */
#ifndef RNNG_MPI_SHIM_H_
#define RNNG_MPI_SHIM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rnng_mpi_type_s* MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_Request;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef long MPI_Aint;
typedef struct rnng_mpi_file_s* MPI_File;

typedef struct MPI_Status {
    int MPI_SOURCE;
    int MPI_TAG;
    int MPI_ERROR;
    long long count_bytes;
} MPI_Status;

/* built-in datatypes (defined in mpi_shim.cpp) */
extern struct rnng_mpi_type_s rnng_mpi_char, rnng_mpi_signed_char, rnng_mpi_short, rnng_mpi_int,
    rnng_mpi_long, rnng_mpi_long_long, rnng_mpi_unsigned_char, rnng_mpi_unsigned_short,
    rnng_mpi_unsigned, rnng_mpi_unsigned_long, rnng_mpi_unsigned_long_long, rnng_mpi_float,
    rnng_mpi_double, rnng_mpi_long_double, rnng_mpi_cxx_bool, rnng_mpi_byte, rnng_mpi_int64_t,
    rnng_mpi_offset;

#define MPI_CHAR               (&rnng_mpi_char)
#define MPI_SIGNED_CHAR        (&rnng_mpi_signed_char)
#define MPI_SHORT              (&rnng_mpi_short)
#define MPI_INT                (&rnng_mpi_int)
#define MPI_LONG               (&rnng_mpi_long)
#define MPI_LONG_LONG          (&rnng_mpi_long_long)
#define MPI_UNSIGNED_CHAR      (&rnng_mpi_unsigned_char)
#define MPI_UNSIGNED_SHORT     (&rnng_mpi_unsigned_short)
#define MPI_UNSIGNED           (&rnng_mpi_unsigned)
#define MPI_UNSIGNED_LONG      (&rnng_mpi_unsigned_long)
#define MPI_UNSIGNED_LONG_LONG (&rnng_mpi_unsigned_long_long)
#define MPI_FLOAT              (&rnng_mpi_float)
#define MPI_DOUBLE             (&rnng_mpi_double)
#define MPI_LONG_DOUBLE        (&rnng_mpi_long_double)
#define MPI_CXX_BOOL           (&rnng_mpi_cxx_bool)
#define MPI_BYTE               (&rnng_mpi_byte)
#define MPI_INT64_T            (&rnng_mpi_int64_t)
#define MPI_OFFSET             (&rnng_mpi_offset)

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

#define MPI_MODE_RDONLY 2
#define MPI_MODE_RDWR   8
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1

#define MPI_IN_PLACE        ((void*)1)
#define MPI_STATUS_IGNORE   ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm* newcomm);
int MPI_Comm_free(MPI_Comm* comm);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
double MPI_Wtime(void);
int MPI_Barrier(MPI_Comm comm);

int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype* newtype);
int MPI_Type_create_resized(MPI_Datatype oldtype, MPI_Aint lb, MPI_Aint extent, MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* datatype);
int MPI_Type_free(MPI_Datatype* datatype);
int MPI_Type_size(MPI_Datatype datatype, int* size);

int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op op, int root, MPI_Comm comm);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op op, MPI_Comm comm);
int MPI_Bcast(void* buffer, int count, MPI_Datatype dt, int root, MPI_Comm comm);
int MPI_Exscan(const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op op, MPI_Comm comm);
int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                  MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Allgatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                   const int* recvcounts, const int* displs, MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
               MPI_Datatype recvtype, int root, MPI_Comm comm);
int MPI_Gatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf,
                const int* recvcounts, const int* displs, MPI_Datatype recvtype, int root, MPI_Comm comm);
int MPI_Alltoall(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                 MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Alltoallv(const void* sendbuf, const int* sendcounts, const int* sdispls, MPI_Datatype sendtype,
                  void* recvbuf, const int* recvcounts, const int* rdispls, MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Ialltoallv(const void* sendbuf, const int* sendcounts, const int* sdispls, MPI_Datatype sendtype,
                   void* recvbuf, const int* recvcounts, const int* rdispls, MPI_Datatype recvtype,
                   MPI_Comm comm, MPI_Request* request);

int MPI_Isend(const void* buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Irecv(void* buf, int count, MPI_Datatype dt, int source, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status* statuses);

int MPI_File_open(MPI_Comm comm, const char* filename, int amode, MPI_Info info, MPI_File* fh);
int MPI_File_close(MPI_File* fh);
int MPI_File_get_size(MPI_File fh, MPI_Offset* size);
int MPI_File_set_size(MPI_File fh, MPI_Offset size);
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype, MPI_Datatype filetype,
                      const char* datarep, MPI_Info info);
int MPI_File_read(MPI_File fh, void* buf, int count, MPI_Datatype dt, MPI_Status* status);
int MPI_File_write_at_all(MPI_File fh, MPI_Offset offset, const void* buf, int count, MPI_Datatype dt,
                          MPI_Status* status);

#ifdef __cplusplus
}
#endif

#endif /* RNNG_MPI_SHIM_H_ */
