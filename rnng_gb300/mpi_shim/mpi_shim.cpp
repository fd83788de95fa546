// Single-rank implementation of the MPI subset declared in mpi.h.
//
// Every communicator has one rank.  Collectives reduce to copies, point-to-point
// messages to self are matched by tag, and MPI-IO is POSIX file I/O with the
// view (displacement + resized file type extent) that RNNG's fvecs reader sets
// up (include/point.hpp:236-271 in RNNG).  Errors print a message and abort,
// which matches RNNG's assert-only error convention (include/utils.h:4).
#include "mpi.h"

#include <fcntl.h>
#include <sys/stat.h>
#include <sys/time.h>
#include <unistd.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <vector>

struct rnng_mpi_type_s {
    long long size;    // bytes of data in one element
    long long extent;  // stride between consecutive elements
    int builtin;
};

#define RNNG_BUILTIN(name, T) struct rnng_mpi_type_s name = {sizeof(T), sizeof(T), 1}
extern "C" {
RNNG_BUILTIN(rnng_mpi_char, char);
RNNG_BUILTIN(rnng_mpi_signed_char, signed char);
RNNG_BUILTIN(rnng_mpi_short, short);
RNNG_BUILTIN(rnng_mpi_int, int);
RNNG_BUILTIN(rnng_mpi_long, long);
RNNG_BUILTIN(rnng_mpi_long_long, long long);
RNNG_BUILTIN(rnng_mpi_unsigned_char, unsigned char);
RNNG_BUILTIN(rnng_mpi_unsigned_short, unsigned short);
RNNG_BUILTIN(rnng_mpi_unsigned, unsigned);
RNNG_BUILTIN(rnng_mpi_unsigned_long, unsigned long);
RNNG_BUILTIN(rnng_mpi_unsigned_long_long, unsigned long long);
RNNG_BUILTIN(rnng_mpi_float, float);
RNNG_BUILTIN(rnng_mpi_double, double);
RNNG_BUILTIN(rnng_mpi_long_double, long double);
RNNG_BUILTIN(rnng_mpi_cxx_bool, bool);
RNNG_BUILTIN(rnng_mpi_byte, unsigned char);
RNNG_BUILTIN(rnng_mpi_int64_t, int64_t);
RNNG_BUILTIN(rnng_mpi_offset, long long);
}

struct rnng_mpi_file_s {
    int fd;
    MPI_Offset disp;       // view displacement in bytes
    long long etype_size;  // bytes per element of the view's etype
    long long ftype_size;  // data bytes per file-type element
    long long ftype_extent;
    MPI_Offset pos;        // individual file pointer, in etypes relative to the view
};

static void shim_fail(const char* what)
{
    std::fprintf(stderr, "mpi shim: %s\n", what);
    std::fflush(stderr);
    std::abort();
}

static long long bytes_of(int count, MPI_Datatype dt)
{
    if (count < 0) shim_fail("negative count");
    return (long long)count * dt->size;
}

static void copy_typed(void* dst, const void* src, int count, MPI_Datatype dt)
{
    if (dst == MPI_IN_PLACE || src == MPI_IN_PLACE || dst == src) return;
    long long n = bytes_of(count, dt);
    if (n > 0) std::memmove(dst, src, (size_t)n);
}

static void check_rank(int r)
{
    if (r != 0) shim_fail("rank other than 0 addressed in a single-rank job");
}

extern "C" {

int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm* newcomm) { *newcomm = comm; return MPI_SUCCESS; }
int MPI_Comm_free(MPI_Comm*) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm, int* rank) { *rank = 0; return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm, int* size) { *size = 1; return MPI_SUCCESS; }

double MPI_Wtime(void)
{
    struct timeval tv;
    gettimeofday(&tv, nullptr);
    return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}

int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype* newtype)
{
    auto* t = new rnng_mpi_type_s;
    t->size = (long long)count * oldtype->size;
    t->extent = (long long)count * oldtype->extent;
    t->builtin = 0;
    *newtype = t;
    return MPI_SUCCESS;
}

int MPI_Type_create_resized(MPI_Datatype oldtype, MPI_Aint lb, MPI_Aint extent, MPI_Datatype* newtype)
{
    if (lb != 0) shim_fail("non-zero lower bound in MPI_Type_create_resized");
    auto* t = new rnng_mpi_type_s;
    t->size = oldtype->size;
    t->extent = extent;
    t->builtin = 0;
    *newtype = t;
    return MPI_SUCCESS;
}

int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }

int MPI_Type_free(MPI_Datatype* dt)
{
    if (dt && *dt && !(*dt)->builtin) delete *dt;
    if (dt) *dt = nullptr;
    return MPI_SUCCESS;
}

int MPI_Type_size(MPI_Datatype dt, int* size) { *size = (int)dt->size; return MPI_SUCCESS; }

int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op, int root, MPI_Comm)
{
    check_rank(root);
    copy_typed(recvbuf, sendbuf, count, dt);
    return MPI_SUCCESS;
}

int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype dt, MPI_Op, MPI_Comm)
{
    copy_typed(recvbuf, sendbuf, count, dt);
    return MPI_SUCCESS;
}

int MPI_Bcast(void*, int, MPI_Datatype, int root, MPI_Comm) { check_rank(root); return MPI_SUCCESS; }

int MPI_Exscan(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm) { return MPI_SUCCESS; }

int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int, MPI_Datatype,
                  MPI_Comm)
{
    copy_typed(recvbuf, sendbuf, sendcount, sendtype);
    return MPI_SUCCESS;
}

int MPI_Allgatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, const int*,
                   const int* displs, MPI_Datatype recvtype, MPI_Comm)
{
    if (sendbuf == MPI_IN_PLACE) return MPI_SUCCESS;
    copy_typed((char*)recvbuf + (long long)displs[0] * recvtype->extent, sendbuf, sendcount, sendtype);
    return MPI_SUCCESS;
}

int MPI_Gather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int, MPI_Datatype,
               int root, MPI_Comm)
{
    check_rank(root);
    copy_typed(recvbuf, sendbuf, sendcount, sendtype);
    return MPI_SUCCESS;
}

int MPI_Gatherv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, const int*,
                const int* displs, MPI_Datatype recvtype, int root, MPI_Comm)
{
    check_rank(root);
    if (sendbuf == MPI_IN_PLACE) return MPI_SUCCESS;
    copy_typed((char*)recvbuf + (long long)displs[0] * recvtype->extent, sendbuf, sendcount, sendtype);
    return MPI_SUCCESS;
}

int MPI_Alltoall(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int, MPI_Datatype,
                 MPI_Comm)
{
    copy_typed(recvbuf, sendbuf, sendcount, sendtype);
    return MPI_SUCCESS;
}

int MPI_Alltoallv(const void* sendbuf, const int* sendcounts, const int* sdispls, MPI_Datatype sendtype,
                  void* recvbuf, const int*, const int* rdispls, MPI_Datatype recvtype, MPI_Comm)
{
    copy_typed((char*)recvbuf + (long long)rdispls[0] * recvtype->extent,
               (const char*)sendbuf + (long long)sdispls[0] * sendtype->extent, sendcounts[0], sendtype);
    return MPI_SUCCESS;
}

// Requests: every non-blocking operation completes when it is matched (sends and
// receives to self) or immediately (collectives).  A request still pending at
// MPI_Waitall is an unmatched message, which cannot complete in a one-rank job.
struct PendingMsg {
    void* buf;
    const void* cbuf;
    long long bytes;
    int req;
};

static std::map<int, std::vector<PendingMsg>> g_sends, g_recvs;
static std::map<int, bool> g_done;
static int g_next_req = 1;

static int new_request(bool done)
{
    int r = g_next_req++;
    g_done[r] = done;
    return r;
}

int MPI_Ialltoallv(const void* sendbuf, const int* sendcounts, const int* sdispls, MPI_Datatype sendtype,
                   void* recvbuf, const int* recvcounts, const int* rdispls, MPI_Datatype recvtype,
                   MPI_Comm comm, MPI_Request* request)
{
    MPI_Alltoallv(sendbuf, sendcounts, sdispls, sendtype, recvbuf, recvcounts, rdispls, recvtype, comm);
    *request = new_request(true);
    return MPI_SUCCESS;
}

int MPI_Isend(const void* buf, int count, MPI_Datatype dt, int dest, int tag, MPI_Comm, MPI_Request* req)
{
    check_rank(dest);
    long long bytes = bytes_of(count, dt);
    auto& rq = g_recvs[tag];
    if (!rq.empty()) {
        PendingMsg r = rq.front();
        rq.erase(rq.begin());
        if (r.bytes < bytes) shim_fail("message truncated");
        if (bytes > 0) std::memcpy(r.buf, buf, (size_t)bytes);
        g_done[r.req] = true;
        *req = new_request(true);
    } else {
        *req = new_request(false);
        g_sends[tag].push_back({nullptr, buf, bytes, *req});
    }
    return MPI_SUCCESS;
}

int MPI_Irecv(void* buf, int count, MPI_Datatype dt, int source, int tag, MPI_Comm, MPI_Request* req)
{
    check_rank(source);
    long long bytes = bytes_of(count, dt);
    auto& sq = g_sends[tag];
    if (!sq.empty()) {
        PendingMsg s = sq.front();
        sq.erase(sq.begin());
        if (bytes < s.bytes) shim_fail("message truncated");
        if (s.bytes > 0) std::memcpy(buf, s.cbuf, (size_t)s.bytes);
        g_done[s.req] = true;
        *req = new_request(true);
    } else {
        *req = new_request(false);
        g_recvs[tag].push_back({buf, nullptr, bytes, *req});
    }
    return MPI_SUCCESS;
}

int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status*)
{
    for (int i = 0; i < count; ++i) {
        auto it = g_done.find(reqs[i]);
        if (it == g_done.end()) continue;  // already completed and released
        if (!it->second) shim_fail("MPI_Waitall on a message with no matching partner (single rank)");
        g_done.erase(it);
    }
    return MPI_SUCCESS;
}

int MPI_File_open(MPI_Comm, const char* filename, int amode, MPI_Info, MPI_File* fh)
{
    int flags = 0;
    if (amode & MPI_MODE_RDWR) flags = O_RDWR;
    else if (amode & MPI_MODE_WRONLY) flags = O_WRONLY;
    else flags = O_RDONLY;
    if (amode & MPI_MODE_CREATE) flags |= O_CREAT;
    int fd = open(filename, flags, 0644);
    if (fd < 0) {
        std::fprintf(stderr, "mpi shim: cannot open '%s'\n", filename);
        std::abort();
    }
    auto* f = new rnng_mpi_file_s;
    f->fd = fd;
    f->disp = 0;
    f->etype_size = 1;
    f->ftype_size = 1;
    f->ftype_extent = 1;
    f->pos = 0;
    *fh = f;
    return MPI_SUCCESS;
}

int MPI_File_close(MPI_File* fh)
{
    if (fh && *fh) {
        close((*fh)->fd);
        delete *fh;
        *fh = nullptr;
    }
    return MPI_SUCCESS;
}

int MPI_File_get_size(MPI_File fh, MPI_Offset* size)
{
    struct stat st;
    if (fstat(fh->fd, &st) != 0) shim_fail("fstat failed");
    *size = (MPI_Offset)st.st_size;
    return MPI_SUCCESS;
}

int MPI_File_set_size(MPI_File fh, MPI_Offset size)
{
    if (ftruncate(fh->fd, (off_t)size) != 0) shim_fail("ftruncate failed");
    return MPI_SUCCESS;
}

int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype, MPI_Datatype filetype, const char*,
                      MPI_Info)
{
    fh->disp = disp;
    fh->etype_size = etype->size;
    fh->ftype_size = filetype->size;
    fh->ftype_extent = filetype->extent;
    fh->pos = 0;
    return MPI_SUCCESS;
}

// Maps a byte position inside the view's data stream to a file offset: data
// bytes come in blocks of ftype_size, one block per ftype_extent of file.
static off_t view_offset(MPI_File fh, long long data_byte)
{
    long long block = data_byte / fh->ftype_size;
    long long within = data_byte % fh->ftype_size;
    return (off_t)(fh->disp + block * fh->ftype_extent + within);
}

static void view_io(MPI_File fh, long long data_byte, char* buf, long long bytes, bool write)
{
    const bool contiguous = (fh->ftype_extent == fh->ftype_size);
    while (bytes > 0) {
        long long within = data_byte % fh->ftype_size;
        long long chunk = contiguous ? bytes : fh->ftype_size - within;
        if (chunk > bytes) chunk = bytes;
        off_t off = view_offset(fh, data_byte);
        long long done = 0;
        while (done < chunk) {
            ssize_t r = write ? pwrite(fh->fd, buf + done, (size_t)(chunk - done), off + done)
                              : pread(fh->fd, buf + done, (size_t)(chunk - done), off + done);
            if (r <= 0) shim_fail(write ? "pwrite failed" : "pread hit end of file");
            done += r;
        }
        buf += chunk;
        data_byte += chunk;
        bytes -= chunk;
    }
}

int MPI_File_read(MPI_File fh, void* buf, int count, MPI_Datatype dt, MPI_Status*)
{
    long long bytes = bytes_of(count, dt);
    view_io(fh, fh->pos * fh->etype_size, (char*)buf, bytes, false);
    fh->pos += bytes / fh->etype_size;
    return MPI_SUCCESS;
}

int MPI_File_write_at_all(MPI_File fh, MPI_Offset offset, const void* buf, int count, MPI_Datatype dt,
                          MPI_Status*)
{
    long long bytes = bytes_of(count, dt);
    view_io(fh, offset * fh->etype_size, (char*)buf, bytes, true);
    return MPI_SUCCESS;
}

}  // extern "C"
