/*
 * Single-rank MPI stand-in used only to build the FargoCPT reference in this
 * repository's oracle recipe (oracle/ref/Makefile).  It is test
 * infrastructure: the GPU engine never includes it.
 *
 * Semantics: one process, rank 0 of a world of size 1.  Collectives copy the
 * send buffer into the receive buffer, point-to-point calls abort (they are
 * unreachable on one rank in the reference: commbound.cpp guards every
 * exchange with CPU_Rank/CPU_Highest checks), and MPI-IO maps onto stdio with
 * the view's displacement and elementary-type size applied to seeks.
 */
#ifndef FARGO_ORACLE_MPI_STUB_H
#define FARGO_ORACLE_MPI_STUB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Request;
typedef long MPI_Aint;
typedef long long MPI_Offset;

typedef struct mpistub_datatype {
    size_t size;
    const char *name;
} *MPI_Datatype;

typedef struct MPI_Status {
    int MPI_SOURCE;
    int MPI_TAG;
    int MPI_ERROR;
    long long count_bytes;
} MPI_Status;

typedef struct mpistub_file *MPI_File;

extern struct mpistub_datatype mpistub_double, mpistub_int, mpistub_unsigned,
    mpistub_unsigned_long, mpistub_char, mpistub_aint, mpistub_int32,
    mpistub_uint32;

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15

#define MPI_DOUBLE (&mpistub_double)
#define MPI_INT (&mpistub_int)
#define MPI_UNSIGNED (&mpistub_unsigned)
#define MPI_UNSIGNED_LONG (&mpistub_unsigned_long)
#define MPI_CHAR (&mpistub_char)
#define MPI_AINT (&mpistub_aint)
#define MPI_INT32_T (&mpistub_int32)
#define MPI_UINT32_T (&mpistub_uint32)

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3

#define MPI_THREAD_SINGLE 0
#define MPI_THREAD_FUNNELED 1
#define MPI_THREAD_SERIALIZED 2
#define MPI_THREAD_MULTIPLE 3

#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1
#define MPI_MODE_APPEND 128

#define MPI_SEEK_SET 600
#define MPI_SEEK_CUR 602
#define MPI_SEEK_END 604

#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_MAX_ERROR_STRING 256
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

int MPI_Init_thread(int *argc, char ***argv, int required, int *provided);
int MPI_Initialized(int *flag);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Barrier(MPI_Comm comm);
int MPI_Get_processor_name(char *name, int *len);
int MPI_Error_string(int code, char *str, int *len);
int MPI_Error_class(int code, int *cls);

int MPI_Allreduce(const void *sbuf, void *rbuf, int count, MPI_Datatype t,
		  MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void *sbuf, void *rbuf, int count, MPI_Datatype t,
	       MPI_Op op, int root, MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm);
int MPI_Gather(const void *sbuf, int scount, MPI_Datatype st, void *rbuf,
	       int rcount, MPI_Datatype rt, int root, MPI_Comm comm);
int MPI_Gatherv(const void *sbuf, int scount, MPI_Datatype st, void *rbuf,
		const int *rcounts, const int *displs, MPI_Datatype rt,
		int root, MPI_Comm comm);
int MPI_Allgather(const void *sbuf, int scount, MPI_Datatype st, void *rbuf,
		  int rcount, MPI_Datatype rt, MPI_Comm comm);

int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag,
	     MPI_Comm comm);
int MPI_Ssend(const void *buf, int count, MPI_Datatype t, int dest, int tag,
	      MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag,
	     MPI_Comm comm, MPI_Status *st);
int MPI_Isend(const void *buf, int count, MPI_Datatype t, int dest, int tag,
	      MPI_Comm comm, MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype t, int src, int tag,
	      MPI_Comm comm, MPI_Request *req);
int MPI_Wait(MPI_Request *req, MPI_Status *st);
int MPI_Probe(int src, int tag, MPI_Comm comm, MPI_Status *st);
int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *count);

int MPI_Get_address(const void *loc, MPI_Aint *addr);
int MPI_Type_create_struct(int count, const int *blocklens,
			   const MPI_Aint *displs, const MPI_Datatype *types,
			   MPI_Datatype *newtype);
int MPI_Type_indexed(int count, const int *blocklens, const int *displs,
		     MPI_Datatype old, MPI_Datatype *newtype);
int MPI_Type_commit(MPI_Datatype *t);
int MPI_Type_free(MPI_Datatype *t);

int MPI_File_open(MPI_Comm comm, const char *name, int amode, MPI_Info info,
		  MPI_File *fh);
int MPI_File_close(MPI_File *fh);
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype,
		      MPI_Datatype ftype, const char *datarep, MPI_Info info);
int MPI_File_seek(MPI_File fh, MPI_Offset offset, int whence);
int MPI_File_write(MPI_File fh, const void *buf, int count, MPI_Datatype t,
		   MPI_Status *st);
int MPI_File_write_all(MPI_File fh, const void *buf, int count,
		       MPI_Datatype t, MPI_Status *st);
int MPI_File_read_all(MPI_File fh, void *buf, int count, MPI_Datatype t,
		      MPI_Status *st);
int MPI_File_get_size(MPI_File fh, MPI_Offset *size);

#ifdef __cplusplus
}
#endif

#endif
