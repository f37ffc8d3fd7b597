/*
 * Single-rank MPI stand-in used only to compile the reference PARENT sources
 * into oracle/_ref/ (test infrastructure, never linked into the product).
 *
 * With one rank every send/receive loop in the reference skips itself
 * (each loop guards on k != rank), so only the calls below are reached:
 * init/finalize, rank/size queries, barriers, broadcasts from rank 0 and abort.
 * Send/Recv are defined so the sources compile; reaching one is a bug and aborts.
 */
#ifndef ORACLE_MPI_STUB_H
#define ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_THREAD_SERIALIZED 2
#define MPI_MAX_PROCESSOR_NAME 64

static inline int MPI_Init_thread(int *, char ***, int req, int *prov) { *prov = req; return 0; }
static inline int MPI_Query_thread(int *prov) { *prov = MPI_THREAD_SERIALIZED; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
static inline int MPI_Get_processor_name(char *n, int *len) {
    strcpy(n, "localhost"); *len = 9; return 0;
}
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { fflush(stdout); exit(code ? code : 1); }
static inline int MPI_Send(const void *, int, MPI_Datatype, int, int, MPI_Comm) {
    fprintf(stderr, "mpi stub: MPI_Send reached with one rank\n"); abort();
}
static inline int MPI_Recv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status *) {
    fprintf(stderr, "mpi stub: MPI_Recv reached with one rank\n"); abort();
}

#endif
