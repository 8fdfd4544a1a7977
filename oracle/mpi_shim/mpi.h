/*
 * Single-rank MPI stand-in used ONLY to compile the reference MITHRA sources as a
 * test oracle (oracle/_ref).  It is test infrastructure, never part of the product.
 *
 * The reference calls a small MPI surface (see the call sites in
 * src/solver.cpp:49-56, :303, :362-365, :458-465, :1552-1572, src/fdtd.cpp:202-209,
 * :728-799, src/radiation.cpp:218).  With one rank:
 *   - rank 0 of size 1;
 *   - reductions copy send to receive (MPI_IN_PLACE is a no-op);
 *   - broadcasts are no-ops;
 *   - point-to-point messages go to a tag-matched self queue, which
 *     Solver::bunchUpdate needs even with one rank (it sends the particles that
 *     crossed a z face to rankB = rankF = 0 and receives them back).
 * A datatype is represented by its size in bytes.
 */
#ifndef MITHRA_ORACLE_MPI_SHIM_H
#define MITHRA_ORACLE_MPI_SHIM_H

#include <string.h>
#include <stdlib.h>

#ifdef __cplusplus
#include <deque>
#include <vector>
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef struct { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; long bytes; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE ((MPI_Datatype)8)
#define MPI_FLOAT ((MPI_Datatype)4)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_IN_PLACE ((void*)1)
#define MPI_SUCCESS 0

#ifdef __cplusplus
namespace mithra_mpi_shim {
struct Message { int tag; std::vector<char> data; };
inline std::deque<Message>& queue() { static std::deque<Message> q; return q; }
}

inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
inline int MPI_Finalize() { return MPI_SUCCESS; }
inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return MPI_SUCCESS; }
inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* t) { *t = count * old; return MPI_SUCCESS; }
inline int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }
inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }

inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != MPI_IN_PLACE && n > 0) memcpy(r, s, (size_t)n * (size_t)t);
  return MPI_SUCCESS;
}
inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  if (s != MPI_IN_PLACE && n > 0) memcpy(r, s, (size_t)n * (size_t)t);
  return MPI_SUCCESS;
}
inline int MPI_Send(const void* buf, int n, MPI_Datatype t, int, int tag, MPI_Comm) {
  mithra_mpi_shim::Message m; m.tag = tag;
  size_t bytes = (size_t)(n > 0 ? n : 0) * (size_t)t;
  m.data.resize(bytes);
  if (bytes) memcpy(m.data.data(), buf, bytes);
  mithra_mpi_shim::queue().push_back(m);
  return MPI_SUCCESS;
}
inline int MPI_Probe(int, int tag, MPI_Comm, MPI_Status* st) {
  for (auto& m : mithra_mpi_shim::queue())
    if (m.tag == tag) { st->MPI_TAG = tag; st->MPI_SOURCE = 0; st->MPI_ERROR = 0; st->bytes = (long)m.data.size(); return MPI_SUCCESS; }
  abort();  /* a receive with no matching send would block forever with one rank */
}
inline int MPI_Get_count(const MPI_Status* st, MPI_Datatype t, int* n) { *n = (int)(st->bytes / t); return MPI_SUCCESS; }
inline int MPI_Recv(void* buf, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Status* st) {
  auto& q = mithra_mpi_shim::queue();
  for (auto it = q.begin(); it != q.end(); ++it)
    if (it->tag == tag) {
      size_t want = (size_t)(n > 0 ? n : 0) * (size_t)t;
      size_t got = it->data.size() < want ? it->data.size() : want;
      if (got) memcpy(buf, it->data.data(), got);
      if (st) { st->MPI_TAG = tag; st->MPI_SOURCE = 0; st->MPI_ERROR = 0; st->bytes = (long)got; }
      q.erase(it);
      return MPI_SUCCESS;
    }
  abort();
}
#endif
#endif
