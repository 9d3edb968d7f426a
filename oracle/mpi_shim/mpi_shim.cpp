// The single-process MPI subset of mpi.h (TEST INFRASTRUCTURE for oracle/_ref; see the
// header for what is restated and from where). Datatypes are type maps: a list of (byte
// displacement, byte length) blocks, a lower bound and an extent; sending packs the blocks
// of each item in order, receiving unpacks into the receiver's blocks in order.
#include "mpi.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <utility>
#include <vector>

namespace {

struct TypeMap {
  std::vector<std::pair<MPI_Aint, MPI_Aint>> blocks;  // (displacement, length) in bytes
  MPI_Aint lb = 0, extent = 0, size = 0;
  bool live = false;
};

std::vector<TypeMap>& types() {
  static std::vector<TypeMap> t = [] {
    std::vector<TypeMap> v(4);
    auto basic = [&](int id, MPI_Aint bytes) {
      v[id].blocks = {{0, bytes}};
      v[id].extent = v[id].size = bytes;
      v[id].live = true;
    };
    basic(MPI_C_DOUBLE_COMPLEX, 16);
    basic(MPI_DOUBLE, 8);
    basic(MPI_INT, 4);
    return v;
  }();
  return t;
}

[[noreturn]] void fail(const char* what) {
  std::fprintf(stderr, "mpi shim: %s\n", what);
  std::abort();
}

const TypeMap& type(MPI_Datatype t) {
  if (t <= 0 || t >= (int)types().size() || !types()[t].live) fail("invalid datatype");
  return types()[t];
}

MPI_Datatype add(TypeMap&& m) {
  m.live = true;
  m.size = 0;
  for (auto& b : m.blocks) m.size += b.second;
  types().push_back(std::move(m));
  return (MPI_Datatype)types().size() - 1;
}

// Appends the blocks of `src` shifted by `shift`, merging with the last block when adjacent.
void append(std::vector<std::pair<MPI_Aint, MPI_Aint>>& dst, const TypeMap& src, MPI_Aint shift) {
  for (auto& b : src.blocks) {
    const MPI_Aint d = b.first + shift;
    if (!dst.empty() && dst.back().first + dst.back().second == d)
      dst.back().second += b.second;
    else
      dst.push_back({d, b.second});
  }
}

// Packs `count` items of type t found at buf.
std::vector<char> pack(const void* buf, int count, MPI_Datatype t) {
  const TypeMap& m = type(t);
  std::vector<char> out((std::size_t)(m.size * count));
  char* o = out.data();
  for (int i = 0; i < count; ++i)
    for (auto& b : m.blocks) {
      std::memcpy(o, static_cast<const char*>(buf) + i * m.extent + b.first, (std::size_t)b.second);
      o += b.second;
    }
  return out;
}

// Unpacks a packed stream into `count` items of type t at buf (the stream must match).
void unpack(const std::vector<char>& in, void* buf, int count, MPI_Datatype t) {
  const TypeMap& m = type(t);
  if ((MPI_Aint)in.size() != m.size * count) fail("message and receive type signatures differ in size");
  const char* s = in.data();
  for (int i = 0; i < count; ++i)
    for (auto& b : m.blocks) {
      std::memcpy(static_cast<char*>(buf) + i * m.extent + b.first, s, (std::size_t)b.second);
      s += b.second;
    }
}

std::deque<std::vector<char>>& mailbox() {
  static std::deque<std::vector<char>> q;
  return q;
}

int next_comm = 2;

}  // namespace

int MPI_Init(int*, char***) { return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm comm, int* rank) {
  if (comm == MPI_COMM_NULL) fail("rank of MPI_COMM_NULL");
  *rank = 0;
  return MPI_SUCCESS;
}
int MPI_Comm_size(MPI_Comm comm, int* size) {
  if (comm == MPI_COMM_NULL) fail("size of MPI_COMM_NULL");
  *size = 1;
  return MPI_SUCCESS;
}
int MPI_Comm_split(MPI_Comm, int, int, MPI_Comm* newcomm) {
  *newcomm = next_comm++;
  return MPI_SUCCESS;
}
int MPI_Comm_free(MPI_Comm* comm) {
  *comm = MPI_COMM_NULL;
  return MPI_SUCCESS;
}
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

int MPI_Type_contiguous(int count, MPI_Datatype oldtype, MPI_Datatype* newtype) {
  const TypeMap old = type(oldtype);
  TypeMap m;
  for (int i = 0; i < count; ++i) append(m.blocks, old, i * old.extent);
  m.lb = old.lb;
  m.extent = count * old.extent;
  *newtype = add(std::move(m));
  return MPI_SUCCESS;
}

int MPI_Type_vector(int count, int blocklength, int stride, MPI_Datatype oldtype, MPI_Datatype* newtype) {
  const TypeMap old = type(oldtype);
  TypeMap m;
  for (int i = 0; i < count; ++i)
    for (int j = 0; j < blocklength; ++j) append(m.blocks, old, ((MPI_Aint)i * stride + j) * old.extent);
  m.lb = old.lb;
  m.extent = count > 0 ? ((MPI_Aint)(count - 1) * stride + blocklength) * old.extent : 0;
  *newtype = add(std::move(m));
  return MPI_SUCCESS;
}

int MPI_Type_create_resized(MPI_Datatype oldtype, MPI_Aint lb, MPI_Aint extent, MPI_Datatype* newtype) {
  TypeMap m = type(oldtype);
  m.lb = lb;
  m.extent = extent;
  *newtype = add(std::move(m));
  return MPI_SUCCESS;
}

int MPI_Type_commit(MPI_Datatype* type_) {
  type(*type_);
  return MPI_SUCCESS;
}

int MPI_Type_free(MPI_Datatype* type_) {
  if (*type_ > MPI_INT) {
    TypeMap& m = types().at(*type_);
    m.blocks.clear();
    m.blocks.shrink_to_fit();
    m.live = false;
  }
  *type_ = MPI_DATATYPE_NULL;
  return MPI_SUCCESS;
}

int MPI_Alltoallv(const void* sendbuf, const int* sendcounts, const int* sdispls, MPI_Datatype sendtype, void* recvbuf,
                  const int* recvcounts, const int* rdispls, MPI_Datatype recvtype, MPI_Comm) {
  const std::vector<char> msg =
      pack(static_cast<const char*>(sendbuf) + (MPI_Aint)sdispls[0] * type(sendtype).extent, sendcounts[0], sendtype);
  unpack(msg, static_cast<char*>(recvbuf) + (MPI_Aint)rdispls[0] * type(recvtype).extent, recvcounts[0], recvtype);
  return MPI_SUCCESS;
}

int MPI_Scatter(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                MPI_Datatype recvtype, int, MPI_Comm) {
  unpack(pack(sendbuf, sendcount, sendtype), recvbuf, recvcount, recvtype);
  return MPI_SUCCESS;
}

int MPI_Allgather(const void* sendbuf, int sendcount, MPI_Datatype sendtype, void* recvbuf, int recvcount,
                  MPI_Datatype recvtype, MPI_Comm) {
  if (sendbuf == MPI_IN_PLACE) return MPI_SUCCESS;
  unpack(pack(sendbuf, sendcount, sendtype), recvbuf, recvcount, recvtype);
  return MPI_SUCCESS;
}

int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype datatype, MPI_Op, MPI_Comm) {
  if (sendbuf == MPI_IN_PLACE) return MPI_SUCCESS;
  unpack(pack(sendbuf, count, datatype), recvbuf, count, datatype);
  return MPI_SUCCESS;
}

int MPI_Sendrecv(const void* sendbuf, int sendcount, MPI_Datatype sendtype, int, int, void* recvbuf, int recvcount,
                 MPI_Datatype recvtype, int, int, MPI_Comm, MPI_Status*) {
  unpack(pack(sendbuf, sendcount, sendtype), recvbuf, recvcount, recvtype);
  return MPI_SUCCESS;
}

int MPI_Send(const void* buf, int count, MPI_Datatype datatype, int, int, MPI_Comm) {
  mailbox().push_back(pack(buf, count, datatype));
  return MPI_SUCCESS;
}

int MPI_Isend(const void* buf, int count, MPI_Datatype datatype, int, int, MPI_Comm, MPI_Request* request) {
  mailbox().push_back(pack(buf, count, datatype));
  *request = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}

int MPI_Recv(void* buf, int count, MPI_Datatype datatype, int, int, MPI_Comm, MPI_Status*) {
  if (mailbox().empty()) fail("receive without a matching send (one process)");
  unpack(mailbox().front(), buf, count, datatype);
  mailbox().pop_front();
  return MPI_SUCCESS;
}

int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return MPI_SUCCESS; }
