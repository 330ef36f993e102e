/* Minimal MPI surface (timer + scalar reductions) for compiling DAKC's
 * counting sources on one host; test infrastructure for the oracle. */
#ifndef DK_SHIM_MPI_H
#define DK_SHIM_MPI_H
#ifdef __cplusplus
extern "C" {
#endif
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_UINT64_T 2
#define MPI_LONG_LONG 3
#define MPI_UINT32_T 4
#define MPI_SUM 1
#define MPI_MAX 2
double MPI_Wtime(void);
int MPI_Reduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c);
int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c);
#ifdef __cplusplus
}
#endif
#endif
