/*
 * Minimal process-based MPI replacement used ONLY to compile and run the
 * unmodified PIMD-B++ reference sources as a CPU oracle (test infrastructure,
 * never part of the GPU product).
 *
 * It provides exactly the MPI surface the reference calls (11 functions plus
 * the handle types and constants), see src/pimdb.cpp:32-37,65,
 * src/simulation.cpp:225-226,282-283,302-346,595-596,
 * src/normal_modes.cpp:15-45,83-86, src/observables/observable.cpp:105.
 *
 * Ranks are forked processes that share one anonymous MAP_SHARED region:
 * MPI_Init forks PIMDB_SHIM_NP-1 children (default 1 = single process).
 */
#ifndef PIMDB_ORACLE_MPI_SHIM_H
#define PIMDB_ORACLE_MPI_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Win;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD ((MPI_Comm)1)
#define MPI_DOUBLE ((MPI_Datatype)1)
#define MPI_SUM ((MPI_Op)1)
#define MPI_INFO_NULL ((MPI_Info)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_SUCCESS 0

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Barrier(MPI_Comm comm);
double MPI_Wtime(void);
int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void* recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status* status);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op op,
                  MPI_Comm comm);
int MPI_Win_allocate_shared(MPI_Aint size, int disp_unit, MPI_Info info, MPI_Comm comm, void* baseptr,
                            MPI_Win* win);
int MPI_Win_shared_query(MPI_Win win, int rank, MPI_Aint* size, int* disp_unit, void* baseptr);
int MPI_Win_free(MPI_Win* win);

#ifdef __cplusplus
}
#endif

#endif
