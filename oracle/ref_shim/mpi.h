/*
 * Single-rank stand-in for the MPI subset that PhiNum's hot-path sources use.
 *
 * TEST INFRASTRUCTURE ONLY: this header lets the reference's own C++ files
 * (dynamics.cpp, fieldanalysis.cpp, momentumspace.cpp, islands.cpp, comm.cpp)
 * compile unchanged into the oracle library under oracle/_ref/.  It is never
 * linked into the product.
 *
 * Semantics with one rank (what `mpirun -np 1` gives the reference):
 *   - rank 0, size 1;
 *   - MPI_Isend / MPI_Irecv to self are matched by tag and completed by a
 *     memcpy as soon as both halves are posted (comm.cpp:43-78 posts the
 *     receive first, islands.cpp:293-300 likewise);
 *   - MPI_Reduce copies send to receive (a sum/min/max over one rank);
 *   - MPI_Bcast and MPI_Barrier do nothing.
 */
#ifndef PHN_ORACLE_MPI_SHIM_H
#define PHN_ORACLE_MPI_SHIM_H

#include <cstring>
#include <cstdio>
#include <cstdlib>
#include <vector>

typedef int MPI_Comm;
typedef int MPI_Datatype; /* encodes the element size in bytes */
typedef int MPI_Op;
struct MPI_Status { int MPI_SOURCE, MPI_TAG, MPI_ERROR; };
typedef int MPI_Request; /* index into the pending table, or MPI_REQUEST_NULL */

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_REQUEST_NULL (-1)
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_LONG_DOUBLE ((MPI_Datatype)sizeof(long double))
#define MPI_DOUBLE_COMPLEX ((MPI_Datatype)(2 * sizeof(double)))
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

namespace phn_mpi_shim {
struct Pending {
  int id;
  bool is_send;
  void *buf;
  size_t bytes;
  int tag;
  bool done;
};
inline std::vector<Pending> &table() {
  static std::vector<Pending> t;
  return t;
}
inline int next_id() {
  static int id = 0;
  return id++;
}
/* Post one half of a self-message; complete it if the other half is waiting. */
inline int post(bool is_send, void *buf, size_t bytes, int tag) {
  std::vector<Pending> &t = table();
  for (size_t i = 0; i < t.size(); ++i) {
    Pending &p = t[i];
    if (!p.done && p.is_send != is_send && p.tag == tag) {
      void *dst = is_send ? p.buf : buf;
      const void *src = is_send ? buf : p.buf;
      size_t n = p.bytes < bytes ? p.bytes : bytes;
      if (dst != src) std::memmove(dst, src, n);
      p.done = true;
      Pending q = {next_id(), is_send, buf, bytes, tag, true};
      t.push_back(q);
      return q.id;
    }
  }
  Pending q = {next_id(), is_send, buf, bytes, tag, false};
  t.push_back(q);
  return q.id;
}
/* Complete request `id`: it must have been matched; its entry is dropped. */
inline bool finish(int id) {
  std::vector<Pending> &t = table();
  for (size_t i = 0; i < t.size(); ++i) {
    if (t[i].id == id) {
      if (!t[i].done) return false;
      t.erase(t.begin() + (long)i);
      return true;
    }
  }
  return false;
}
} // namespace phn_mpi_shim

inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
inline int MPI_Finalize() { return MPI_SUCCESS; }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return MPI_SUCCESS; }
/* PHN_SHIM_NODES > 1 reports more ranks (this process stays rank 0), only to
 * check that a caller refuses a multi-rank run before any message is sent. */
#ifndef PHN_SHIM_NODES
#define PHN_SHIM_NODES 1
#endif
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = PHN_SHIM_NODES; return MPI_SUCCESS; }
inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  if (s != r) std::memmove(r, s, (size_t)n * (size_t)t);
  return MPI_SUCCESS;
}
inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *req) {
  *req = phn_mpi_shim::post(true, const_cast<void *>(b), (size_t)n * (size_t)t, tag);
  return MPI_SUCCESS;
}
inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *req) {
  *req = phn_mpi_shim::post(false, b, (size_t)n * (size_t)t, tag);
  return MPI_SUCCESS;
}
inline int MPI_Wait(MPI_Request *req, MPI_Status *) {
  if (*req == MPI_REQUEST_NULL) return MPI_SUCCESS;
  if (!phn_mpi_shim::finish(*req)) {
    std::fprintf(stderr, "mpi shim: wait on an unmatched self-message\n");
    std::abort();
  }
  *req = MPI_REQUEST_NULL;
  return MPI_SUCCESS;
}

#endif
