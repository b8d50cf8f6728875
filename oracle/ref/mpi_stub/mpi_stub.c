/*
 * Single-rank MPI stand-in (see mpi.h for the contract).  Built only by the
 * oracle recipe that compiles the FargoCPT reference for parity fixtures.
 */
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct mpistub_datatype mpistub_double = {sizeof(double), "double"};
struct mpistub_datatype mpistub_int = {sizeof(int), "int"};
struct mpistub_datatype mpistub_unsigned = {sizeof(unsigned), "unsigned"};
struct mpistub_datatype mpistub_unsigned_long = {sizeof(unsigned long),
						 "unsigned long"};
struct mpistub_datatype mpistub_char = {sizeof(char), "char"};
struct mpistub_datatype mpistub_aint = {sizeof(MPI_Aint), "aint"};
struct mpistub_datatype mpistub_int32 = {4, "int32"};
struct mpistub_datatype mpistub_uint32 = {4, "uint32"};

struct mpistub_file {
    FILE *f;
    long long disp;
    size_t esize;
};

static int initialized = 0;

static void unreachable(const char *what)
{
    fprintf(stderr, "mpi stub: %s called on a single rank\n", what);
    abort();
}

static void copy(const void *s, void *r, int count, MPI_Datatype t)
{
    if (s != r && count > 0) {
	memmove(r, s, (size_t)count * t->size);
    }
}

int MPI_Init_thread(int *argc, char ***argv, int required, int *provided)
{
    (void)argc;
    (void)argv;
    *provided = required;
    initialized = 1;
    return MPI_SUCCESS;
}
int MPI_Initialized(int *flag)
{
    *flag = initialized;
    return MPI_SUCCESS;
}
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm comm, int code)
{
    (void)comm;
    exit(code);
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
int MPI_Barrier(MPI_Comm comm)
{
    (void)comm;
    return MPI_SUCCESS;
}
int MPI_Get_processor_name(char *name, int *len)
{
    strcpy(name, "localhost");
    *len = (int)strlen(name);
    return MPI_SUCCESS;
}
int MPI_Error_string(int code, char *str, int *len)
{
    *len = snprintf(str, MPI_MAX_ERROR_STRING, "mpi stub error %d", code);
    return MPI_SUCCESS;
}
int MPI_Error_class(int code, int *cls)
{
    *cls = code;
    return MPI_SUCCESS;
}

int MPI_Allreduce(const void *sbuf, void *rbuf, int count, MPI_Datatype t,
		  MPI_Op op, MPI_Comm comm)
{
    (void)op;
    (void)comm;
    copy(sbuf, rbuf, count, t);
    return MPI_SUCCESS;
}
int MPI_Reduce(const void *sbuf, void *rbuf, int count, MPI_Datatype t,
	       MPI_Op op, int root, MPI_Comm comm)
{
    (void)op;
    (void)root;
    (void)comm;
    copy(sbuf, rbuf, count, t);
    return MPI_SUCCESS;
}
int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm comm)
{
    (void)buf;
    (void)count;
    (void)t;
    (void)root;
    (void)comm;
    return MPI_SUCCESS;
}
int MPI_Gather(const void *sbuf, int scount, MPI_Datatype st, void *rbuf,
	       int rcount, MPI_Datatype rt, int root, MPI_Comm comm)
{
    (void)rcount;
    (void)rt;
    (void)root;
    (void)comm;
    copy(sbuf, rbuf, scount, st);
    return MPI_SUCCESS;
}
int MPI_Gatherv(const void *sbuf, int scount, MPI_Datatype st, void *rbuf,
		const int *rcounts, const int *displs, MPI_Datatype rt,
		int root, MPI_Comm comm)
{
    (void)rcounts;
    (void)root;
    (void)comm;
    copy(sbuf, (char *)rbuf + (size_t)displs[0] * rt->size, scount, st);
    return MPI_SUCCESS;
}
int MPI_Allgather(const void *sbuf, int scount, MPI_Datatype st, void *rbuf,
		  int rcount, MPI_Datatype rt, MPI_Comm comm)
{
    (void)rcount;
    (void)rt;
    (void)comm;
    copy(sbuf, rbuf, scount, st);
    return MPI_SUCCESS;
}

int MPI_Send(const void *b, int c, MPI_Datatype t, int d, int g, MPI_Comm m)
{
    (void)b, (void)c, (void)t, (void)d, (void)g, (void)m;
    unreachable("MPI_Send");
    return MPI_ERR_OTHER;
}
int MPI_Ssend(const void *b, int c, MPI_Datatype t, int d, int g, MPI_Comm m)
{
    (void)b, (void)c, (void)t, (void)d, (void)g, (void)m;
    unreachable("MPI_Ssend");
    return MPI_ERR_OTHER;
}
int MPI_Recv(void *b, int c, MPI_Datatype t, int s, int g, MPI_Comm m,
	     MPI_Status *st)
{
    (void)b, (void)c, (void)t, (void)s, (void)g, (void)m, (void)st;
    unreachable("MPI_Recv");
    return MPI_ERR_OTHER;
}
int MPI_Isend(const void *b, int c, MPI_Datatype t, int d, int g, MPI_Comm m,
	      MPI_Request *r)
{
    (void)b, (void)c, (void)t, (void)d, (void)g, (void)m, (void)r;
    unreachable("MPI_Isend");
    return MPI_ERR_OTHER;
}
int MPI_Irecv(void *b, int c, MPI_Datatype t, int s, int g, MPI_Comm m,
	      MPI_Request *r)
{
    (void)b, (void)c, (void)t, (void)s, (void)g, (void)m, (void)r;
    unreachable("MPI_Irecv");
    return MPI_ERR_OTHER;
}
int MPI_Wait(MPI_Request *r, MPI_Status *st)
{
    (void)r, (void)st;
    unreachable("MPI_Wait");
    return MPI_ERR_OTHER;
}
int MPI_Probe(int s, int g, MPI_Comm m, MPI_Status *st)
{
    (void)s, (void)g, (void)m, (void)st;
    unreachable("MPI_Probe");
    return MPI_ERR_OTHER;
}
int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *count)
{
    *count = (int)(st->count_bytes / (long long)t->size);
    return MPI_SUCCESS;
}

int MPI_Get_address(const void *loc, MPI_Aint *addr)
{
    *addr = (MPI_Aint)loc;
    return MPI_SUCCESS;
}
int MPI_Type_create_struct(int count, const int *blocklens,
			   const MPI_Aint *displs, const MPI_Datatype *types,
			   MPI_Datatype *newtype)
{
    size_t extent = 0;
    for (int i = 0; i < count; ++i) {
	size_t end = (size_t)displs[i] + (size_t)blocklens[i] * types[i]->size;
	if (end > extent) {
	    extent = end;
	}
    }
    struct mpistub_datatype *t = malloc(sizeof(*t));
    t->size = extent;
    t->name = "struct";
    *newtype = t;
    return MPI_SUCCESS;
}
int MPI_Type_indexed(int count, const int *blocklens, const int *displs,
		     MPI_Datatype old, MPI_Datatype *newtype)
{
    size_t extent = 0;
    for (int i = 0; i < count; ++i) {
	size_t end = ((size_t)displs[i] + (size_t)blocklens[i]) * old->size;
	if (end > extent) {
	    extent = end;
	}
    }
    struct mpistub_datatype *t = malloc(sizeof(*t));
    t->size = extent;
    t->name = "indexed";
    *newtype = t;
    return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype *t)
{
    (void)t;
    return MPI_SUCCESS;
}
int MPI_Type_free(MPI_Datatype *t)
{
    (void)t;
    return MPI_SUCCESS;
}

int MPI_File_open(MPI_Comm comm, const char *name, int amode, MPI_Info info,
		  MPI_File *fh)
{
    (void)comm;
    (void)info;
    FILE *f = NULL;
    if (amode & MPI_MODE_RDONLY) {
	f = fopen(name, "rb");
    } else {
	f = fopen(name, "r+b");
	if (f == NULL && (amode & MPI_MODE_CREATE)) {
	    f = fopen(name, "w+b");
	}
	if (f != NULL && (amode & MPI_MODE_APPEND)) {
	    fseek(f, 0, SEEK_END);
	}
    }
    if (f == NULL) {
	*fh = NULL;
	return MPI_ERR_OTHER;
    }
    struct mpistub_file *h = malloc(sizeof(*h));
    h->f = f;
    h->disp = 0;
    h->esize = 1;
    *fh = h;
    return MPI_SUCCESS;
}
int MPI_File_close(MPI_File *fh)
{
    if (*fh) {
	fclose((*fh)->f);
	free(*fh);
	*fh = NULL;
    }
    return MPI_SUCCESS;
}
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype,
		      MPI_Datatype ftype, const char *datarep, MPI_Info info)
{
    (void)ftype;
    (void)datarep;
    (void)info;
    fh->disp = disp;
    fh->esize = etype->size;
    return MPI_SUCCESS;
}
int MPI_File_seek(MPI_File fh, MPI_Offset offset, int whence)
{
    if (whence & (MPI_SEEK_END & ~MPI_SEEK_SET)) {
	fseek(fh->f, 0, SEEK_END);
	return MPI_SUCCESS;
    }
    if (whence == MPI_SEEK_CUR) {
	fseek(fh->f, (long)(offset * (MPI_Offset)fh->esize), SEEK_CUR);
	return MPI_SUCCESS;
    }
    fseek(fh->f, (long)(fh->disp + offset * (MPI_Offset)fh->esize), SEEK_SET);
    return MPI_SUCCESS;
}
int MPI_File_write(MPI_File fh, const void *buf, int count, MPI_Datatype t,
		   MPI_Status *st)
{
    size_t n = fwrite(buf, t->size, (size_t)count, fh->f);
    if (st) {
	st->count_bytes = (long long)(n * t->size);
	st->MPI_ERROR = MPI_SUCCESS;
    }
    return n == (size_t)count ? MPI_SUCCESS : MPI_ERR_OTHER;
}
int MPI_File_write_all(MPI_File fh, const void *buf, int count,
		       MPI_Datatype t, MPI_Status *st)
{
    return MPI_File_write(fh, buf, count, t, st);
}
int MPI_File_read_all(MPI_File fh, void *buf, int count, MPI_Datatype t,
		      MPI_Status *st)
{
    size_t n = fread(buf, t->size, (size_t)count, fh->f);
    if (st) {
	st->count_bytes = (long long)(n * t->size);
	st->MPI_ERROR = MPI_SUCCESS;
    }
    return MPI_SUCCESS;
}
int MPI_File_get_size(MPI_File fh, MPI_Offset *size)
{
    long pos = ftell(fh->f);
    fseek(fh->f, 0, SEEK_END);
    *size = (MPI_Offset)ftell(fh->f);
    fseek(fh->f, pos, SEEK_SET);
    return MPI_SUCCESS;
}
