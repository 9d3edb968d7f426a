// A single-process subset of the MPI interface, so that the reference's own C++ sources
// (which include <mpi.h>) compile and run here as the oracle's cross-check at world size
// 1. TEST INFRASTRUCTURE: used only to build oracle/_ref, never by the product.
//
// MPI itself is not part of the reference (it is a system dependency, unpinned: the README
// asks for "MPI - version 4.1", CMake uses find_package(MPI)). What the reference uses of it
// is restated here from the MPI standard's published semantics (MPI 4.1, chapters 4 and 6):
//   * derived datatypes: MPI_Type_contiguous, MPI_Type_vector, MPI_Type_create_resized
//     describe a type map (byte displacement, length) with a lower bound and an extent; a
//     buffer of `count` items of a type is the type map repeated at multiples of the extent;
//     sender and receiver type maps are matched element by element (the type signature);
//   * communicators of one process: every rank is 0, every size 1, MPI_Comm_split returns
//     a one-process communicator;
//   * collectives and point-to-point calls with oneself: Alltoallv, Scatter, Allgather,
//     Allreduce (MPI_IN_PLACE leaves the buffer as it is), Sendrecv, and Isend + Recv (a
//     queue of packed messages), all as packing the send buffer by its type map and
//     unpacking into the receive buffer by the receiver's.
#ifndef QTNH_ORACLE_MPI_SHIM_H
#define QTNH_ORACLE_MPI_SHIM_H

#include <cstddef>
#include <stdint.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef std::ptrdiff_t MPI_Aint;
struct MPI_Status {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
};

#define MPI_SUCCESS 0
#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_DATATYPE_NULL 0
#define MPI_C_DOUBLE_COMPLEX 1
#define MPI_DOUBLE 2
#define MPI_INT 3
#define MPI_SUM 1
#define MPI_REQUEST_NULL 0
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_split(MPI_Comm comm, int colour, int key, MPI_Comm* newcomm);
int MPI_Comm_free(MPI_Comm* comm);
int MPI_Barrier(MPI_Comm comm);

int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype* newtype);
int MPI_Type_vector(int count, int blocklength, int stride, MPI_Datatype oldtype, MPI_Datatype* newtype);
int MPI_Type_create_resized(MPI_Datatype oldtype, MPI_Aint lb, MPI_Aint extent, MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* type);
int MPI_Type_free(MPI_Datatype* type);

int MPI_Alltoallv(const void* sendbuf, const int* sendcounts, const int* sdispls, MPI_Datatype sendtype, void* recvbuf,
                  const int* recvcounts, const int* rdispls, MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Scatter(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                MPI_Datatype recvtype, int root, MPI_Comm comm);
int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                  MPI_Datatype recvtype, MPI_Comm comm);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op op, MPI_Comm comm);
int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag, void* recvbuf,
                 int recvcount, MPI_Datatype recvtype, int source, int recvtag, MPI_Comm comm, MPI_Status* status);
int MPI_Send(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm);
int MPI_Isend(const void* buf, int count, MPI_Datatype datatype, int dest, int tag, MPI_Comm comm,
              MPI_Request* request);
int MPI_Recv(void* buf, int count, MPI_Datatype datatype, int source, int tag, MPI_Comm comm, MPI_Status* status);
int MPI_Waitall(int count, MPI_Request* requests, MPI_Status* statuses);

#endif
