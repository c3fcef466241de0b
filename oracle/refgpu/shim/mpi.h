/* One-rank MPI declarations for the device build of the reference kernels:
 * the reference headers include <mpi.h> for types the kernels never use. */
#ifndef REFGPU_MPI_H
#define REFGPU_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Win;
typedef int MPI_Request;
typedef int MPI_Group;
typedef int MPI_Info;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_FLOAT 2
#define MPI_INT 3
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_PROC_NULL (-1)
#define MPI_IN_PLACE ((void *)1)
#endif
