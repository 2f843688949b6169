/*
 * mpi.h - single-rank stand-in for the MPI interface the reference's hot-path sources use.
 *
 * TEST INFRASTRUCTURE ONLY: it lets src/Simulation.cpp, src/Domain.cpp, src/MPIDomain.cpp
 * and src/MPIDetails.cpp of the reference compile unchanged into the parity library under
 * oracle/_ref (see oracle/build_ref.py). One process is rank 0 of a communicator of size 1:
 * reductions and broadcasts copy their input, point-to-point calls are never reached (the
 * halo exchange of src/MPIDomain.h:138-165 has no neighbour ranks), MPI_Abort throws.
 * Only what those four files call is declared.
 */
#ifndef LSREF_SHIM_MPI_H_
#define LSREF_SHIM_MPI_H_

#include <stddef.h>
#include <stdint.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef int MPI_File;
typedef long long MPI_Offset;
typedef intptr_t MPI_Aint;
typedef struct MPI_Status {
    int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 4
#define MPI_SEEK_SET 600

enum {
    MPI_CHAR = 1, MPI_UNSIGNED_CHAR, MPI_SHORT, MPI_UNSIGNED_SHORT, MPI_INT, MPI_UNSIGNED, MPI_LONG,
    MPI_UNSIGNED_LONG, MPI_LONG_LONG, MPI_UNSIGNED_LONG_LONG, MPI_FLOAT, MPI_DOUBLE, LSREF_MPI_FIRST_DERIVED
};
enum { MPI_MAX = 1, MPI_MIN, MPI_SUM };
enum {
    MPI_SUCCESS = 0, MPI_ERR_COMM, MPI_ERR_TYPE, MPI_ERR_COUNT, MPI_ERR_TAG, MPI_ERR_RANK, MPI_ERR_IN_STATUS,
    MPI_ERR_OTHER
};

#ifdef __cplusplus
extern "C" {
#endif
int MPI_Initialized(int* flag);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Barrier(MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                  MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Isend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status* statuses);
int MPI_Get_address(const void* location, MPI_Aint* address);
int MPI_Type_create_struct(int count, const int* blocklengths, const MPI_Aint* displacements,
                           const MPI_Datatype* types, MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* type);
int MPI_File_open(MPI_Comm comm, const char* filename, int amode, MPI_Info info, MPI_File* fh);
int MPI_File_seek(MPI_File fh, MPI_Offset offset, int whence);
int MPI_File_write(MPI_File fh, const void* buf, int count, MPI_Datatype type, MPI_Status* status);
int MPI_File_close(MPI_File* fh);
#ifdef __cplusplus
}
#endif

#endif /* LSREF_SHIM_MPI_H_ */
