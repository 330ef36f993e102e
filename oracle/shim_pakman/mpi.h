// One-rank stand-in for the MPI calls PakMan*'s k-mer counting makes
// (pakman_star/src/kmer_counting.cpp), so that those sources compile
// unmodified for the oracle.  With a single rank every collective is a copy.
// Test infrastructure only (oracle/pakman_harness.cpp implements them).
#pragma once
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Comm;
typedef int MPI_File;
#define MPI_COMM_WORLD 0
#define MPI_BYTE 1
#define MPI_INT 4
#define MPI_UINT64_T 8
#define MPI_SUM 0
int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype type, MPI_Op op,
                  MPI_Comm comm);
int MPI_Barrier(MPI_Comm comm);
int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* out);
int MPI_Type_commit(MPI_Datatype* type);
int MPI_Type_free(MPI_Datatype* type);
int MPI_Alltoall(const void* send, int scount, MPI_Datatype stype, void* recv, int rcount,
                 MPI_Datatype rtype, MPI_Comm comm);
int MPI_Alltoallv(const void* send, const int* scounts, const int* sdispls, MPI_Datatype stype,
                  void* recv, const int* rcounts, const int* rdispls, MPI_Datatype rtype,
                  MPI_Comm comm);
