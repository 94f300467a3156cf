/* mpi.h -- single-rank stand-in for the MPI names the reference's reader
 * headers use (src/AdPointDataReaders.h, src/AdLagrangianRedistribution.h,
 * src/AdMeasureMPIWallClockTime.h).  TEST INFRASTRUCTURE ONLY: it lets
 * oracle/ref_readers.cpp compile and run the reference's own readers on one
 * rank so that their output can pin this repository's readers.  With one rank
 * the collectives are copies, the file calls are stdio. */
#ifndef ADECO_ORACLE_MPI_STUB_H
#define ADECO_ORACLE_MPI_STUB_H

#include <cstdio>
#include <cstring>
#include <ctime>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long long MPI_Offset;
struct MPI_Status {
    long long bytes;
};
struct MPI_FileRec {
    std::FILE *f;
    long long disp;
    int esize;
};
typedef MPI_FileRec *MPI_File;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_MODE_RDONLY 1
#define MPI_THREAD_FUNNELED 1
#define MPI_MAX_ERROR_STRING 256
#define MPI_MAX_LIBRARY_VERSION_STRING 256
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
/* datatypes are their sizes in bytes */
#define MPI_CHAR 1
#define MPI_FLOAT 4
#define MPI_DOUBLE 8
#define MPI_LONG_INT 8
#define MPI_LONG_LONG 8
#define MPI_LONG_LONG_INT 8
#define MPI_UNSIGNED_LONG 8
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Init_thread(int *, char ***, int, int *p) { if (p) *p = MPI_THREAD_FUNNELED; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *n) { *n = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm)
{
    if (s != r) std::memcpy(r, s, (size_t)n * (size_t)t);
    return 0;
}
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm)
{
    if (s != r) std::memcpy(r, s, (size_t)n * (size_t)t);
    return 0;
}
static inline int MPI_Allgather(const void *s, int sc, MPI_Datatype st, void *r, int, MPI_Datatype, MPI_Comm)
{
    std::memcpy(r, s, (size_t)sc * (size_t)st);
    return 0;
}
static inline int MPI_Sendrecv(const void *s, int sc, MPI_Datatype st, int, int, void *r, int, MPI_Datatype, int, int,
                               MPI_Comm, MPI_Status *)
{
    std::memcpy(r, s, (size_t)sc * (size_t)st);
    return 0;
}
static inline double MPI_Wtime() { return (double)std::clock() / CLOCKS_PER_SEC; }
static inline int MPI_Error_string(int, char *s, int *n) { s[0] = 0; *n = 0; return 0; }
static inline int MPI_Get_library_version(char *s, int *n) { std::strcpy(s, "single-rank stand-in"); *n = (int)std::strlen(s); return 0; }
static inline int MPI_Get_version(int *v, int *sv) { *v = 3; *sv = 0; return 0; }
static inline int MPI_File_open(MPI_Comm, const char *name, int, MPI_Info, MPI_File *fh)
{
    std::FILE *f = std::fopen(name, "rb");
    if (!f) return 1;
    *fh = new MPI_FileRec{f, 0, 1};
    return 0;
}
static inline int MPI_File_get_size(MPI_File fh, MPI_Offset *sz)
{
    const long cur = std::ftell(fh->f);
    std::fseek(fh->f, 0, SEEK_END);
    *sz = std::ftell(fh->f);
    std::fseek(fh->f, cur, SEEK_SET);
    return 0;
}
static inline int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype, MPI_Datatype, const char *, MPI_Info)
{
    fh->disp = disp;
    fh->esize = etype;
    return std::fseek(fh->f, (long)disp, SEEK_SET);
}
static inline int MPI_File_read(MPI_File fh, void *buf, int count, MPI_Datatype t, MPI_Status *st)
{
    const size_t got = std::fread(buf, (size_t)t, (size_t)count, fh->f);
    if (st) st->bytes = (long long)(got * (size_t)t);
    return got == (size_t)count ? 0 : 1;
}
static inline int MPI_File_read_at(MPI_File fh, MPI_Offset off, void *buf, int count, MPI_Datatype t, MPI_Status *st)
{
    std::fseek(fh->f, (long)(fh->disp + off * fh->esize), SEEK_SET);
    return MPI_File_read(fh, buf, count, t, st);
}
static inline int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *n) { *n = (int)(st->bytes / t); return 0; }
static inline int MPI_File_close(MPI_File *fh)
{
    std::fclose((*fh)->f);
    delete *fh;
    *fh = 0;
    return 0;
}

#endif
