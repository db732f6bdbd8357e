/* Serial stand-in for <mpi.h>, used only to compile the reference's hot-path
 * sources into the single-process oracle build.  Types and no-op calls; the
 * oracle never calls any of them. */
#ifndef ORACLE_SERIAL_MPI_H
#define ORACLE_SERIAL_MPI_H
typedef int MPI_Datatype;
typedef int MPI_Comm;
typedef int MPI_Request;
typedef long MPI_Aint;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_UNSIGNED 2
#define MPI_DOUBLE 3
#define MPI_SUM 0
#define MPI_MIN 1
#define MPI_MAX 2
static inline int MPI_Type_struct(int, int *, MPI_Aint *, MPI_Datatype *, MPI_Datatype *) { return 0; }
static inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
static inline int MPI_Irecv(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return 0; }
static inline int MPI_Isend(void *, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request *) { return 0; }
static inline int MPI_Wait(MPI_Request *, MPI_Status *) { return 0; }
static inline int MPI_Allreduce(void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { return 0; }
static inline int MPI_Abort(MPI_Comm, int) { return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
#endif
