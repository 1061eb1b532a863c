/*
 * Single-rank stand-in for <mpi.h>, used ONLY to compile the reference's own
 * hot-path sources (flood.c, attributes.c, filtering.c, pattern.c, ...) into
 * the test oracle under oracle/_ref/.  This is test infrastructure: nothing in
 * the product links it.
 *
 * Every call behaves as it would in a one-process MPI job: rank 0 of 1,
 * reductions copy their input, datatype constructors are no-ops, MPI_Abort
 * exits.  Only the names the reference's hot-path translation units use are
 * provided (collected from flood.c, attributes.c, filtering.c, pattern.c,
 * queue.c, workspace.c, lambdavec.c, eispack.c, logc.c, checks.c,
 * mpihelper.c, preprocessing.c, operation.c, csl.c and the headers).
 */
#ifndef DCF_ORACLE_MPI_STUB_H
#define DCF_ORACLE_MPI_STUB_H

#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_THREAD_FUNNELED 1
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

/* Datatype handles encode their element size so the single-rank reduce can copy. */
#define MPI_CHAR 1
#define MPI_UINT8_T 1
#define MPI_UINT16_T 2
#define MPI_INT 4
#define MPI_FLOAT 4
#define MPI_UINT32_T 4
#define MPI_UINT 4
#define MPI_DOUBLE 8
#define MPI_INT64_T 8
#define MPI_UINT64_T 8
#define MPI_UNSIGNED_LONG 8
#define MPI_LONG 8

#define MPI_MIN 1
#define MPI_MAX 2
#define MPI_SUM 3

static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *n) { (void)c; *n = 1; return 0; }
static inline int MPI_Initialized(int *f) { *f = 1; return 0; }
static inline int MPI_Finalized(int *f) { *f = 1; return 0; }
static inline int MPI_Init_thread(int *a, char ***b, int req, int *prov) { (void)a; (void)b; *prov = req; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
static inline int MPI_Abort(MPI_Comm c, int code) { (void)c; fprintf(stderr, "MPI_Abort(%d)\n", code); exit(code ? code : 1); }
static inline int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Type_free(MPI_Datatype *t) { (void)t; return 0; }
static inline int MPI_Type_create_struct(int n, const int *bl, const MPI_Aint *off, const MPI_Datatype *ty, MPI_Datatype *out)
{ (void)n; (void)bl; (void)off; (void)ty; *out = 0; return 0; }
static inline int MPI_Type_vector(int c, int bl, int st, MPI_Datatype old, MPI_Datatype *out)
{ (void)c; (void)bl; (void)st; (void)old; *out = 0; return 0; }
static inline int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{ (void)op; (void)c; if (in != out) memcpy(out, in, (size_t)count * (size_t)t); return 0; }
static inline int MPI_Reduce(const void *in, void *out, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c)
{ (void)op; (void)root; (void)c; if (in != out) memcpy(out, in, (size_t)count * (size_t)t); return 0; }
static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; return 0; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; return 0; }

#endif
