// Single-rank stand-in for the MPI header the reference sources include
// (MPI is not installed here).  Declarations only: the reference functions
// pinned by oracle/pins/ecsim_pin.cpp make no MPI call, and the harness links
// with unresolved symbols ignored.
#pragma once
#include <string.h>
typedef int MPI_Comm; typedef int MPI_Datatype; typedef int MPI_Op; typedef int MPI_Request; typedef int MPI_Fint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_LONG 3
#define MPI_CHAR 4
#define MPI_BYTE 5
#define MPI_UNSIGNED_LONG 6
#define MPI_UNSIGNED_CHAR 7
#define MPI_UNSIGNED 8
#define MPI_LONG_LONG 9
#define MPI_FLOAT 10
#define MPI_SHORT 11
#define MPI_SUM 0
#define MPI_MAX 1
#define MPI_MIN 2
#define MPI_LOR 3
#define MPI_LAND 4
#define MPI_SUCCESS 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_ANY_SOURCE -1
#define MPI_ANY_TAG -1
#define MPI_IN_PLACE ((void*)1)
#define MPI_REQUEST_NULL 0
#define MPI_DATATYPE_NULL 0
int MPI_Reduce(const void*, void*, int, MPI_Datatype, MPI_Op, int, MPI_Comm);
int MPI_Allreduce(const void*, void*, int, MPI_Datatype, MPI_Op, MPI_Comm);
int MPI_Allgather(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, MPI_Comm);
int MPI_Gather(const void*, int, MPI_Datatype, void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm);
int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm);
int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*);
int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*);
int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*);
int MPI_Wait(MPI_Request*, MPI_Status*);
int MPI_Waitall(int, MPI_Request*, MPI_Status*);
int MPI_Barrier(MPI_Comm);
int MPI_Comm_rank(MPI_Comm, int*);
int MPI_Comm_size(MPI_Comm, int*);
int MPI_Type_indexed(int, const int*, const int*, MPI_Datatype, MPI_Datatype*);
int MPI_Type_commit(MPI_Datatype*);
int MPI_Type_free(MPI_Datatype*);
MPI_Fint MPI_Comm_c2f(MPI_Comm);
double MPI_Wtime();
int MPI_Abort(MPI_Comm, int);
int MPI_Finalize();
int MPI_Init(int*, char***);
#define MPI_UNDEFINED -32766
#define MPI_UNSIGNED_SHORT 12
#define MPI_LONG_DOUBLE 13
int MPI_Testany(int, MPI_Request*, int*, int*, MPI_Status*);
int MPI_Initialized(int*);
int MPI_Iprobe(int, int, MPI_Comm, int*, MPI_Status*);
