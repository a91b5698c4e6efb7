// Single-rank implementation of the MPI subset declared in include/mpi.h.
// One process, rank 0, size 1.  Cartesian communicators remember their number
// of dimensions so that PFFT's planners can derive the mesh rank from them
// (kernel/procmesh.c:36-64 creates them, kernel/partrafo.c uses
// MPI_Cartdim_get; a non-Cartesian communicator becomes a 1-D mesh,
// kernel/procmesh.c:114-129).
#include <string.h>
#include <time.h>
#include <mutex>
#include <vector>
#include "../../include/mpi.h"
#include "core.h"

namespace {
std::mutex g_mu;
// handle -> Cartesian dimension (0 = plain communicator); handles >= 16 are
// created by MPI_Cart_create / MPI_Comm_dup / MPI_Cart_sub
std::vector<int> g_dims = {-1, 0, 0};  // NULL (invalid), WORLD, SELF
std::vector<char> g_live = {0, 1, 1};
int g_init = 0, g_final = 0;

int new_handle(int dims) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (size_t h = 3; h < g_dims.size(); h++)
    if (!g_live[h]) {
      g_dims[h] = dims;
      g_live[h] = 1;
      return (int)h;
    }
  g_dims.push_back(dims);
  g_live.push_back(1);
  return (int)g_dims.size() - 1;
}

size_t type_size(MPI_Datatype t) {
  switch (t) {
    case MPI_CHAR: case MPI_BYTE: return 1;
    case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: return 4;
    case MPI_LONG: case MPI_DOUBLE: case MPI_LONG_LONG: return 8;
    case MPI_LONG_DOUBLE: return sizeof(long double);
  }
  return 1;
}
}  // namespace

namespace pg {
bool comm_valid(int comm) {
  std::lock_guard<std::mutex> lk(g_mu);
  return comm > 0 && (size_t)comm < g_live.size() && g_live[comm];
}
int comm_cart_dims(int comm) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (comm <= 0 || (size_t)comm >= g_dims.size()) return 0;
  return g_dims[comm] > 0 ? g_dims[comm] : 0;
}
}  // namespace pg

extern "C" {

int MPI_Init(int*, char***) {
  g_init = 1;
  return MPI_SUCCESS;
}
int MPI_Initialized(int* flag) {
  *flag = g_init;
  return MPI_SUCCESS;
}
int MPI_Finalize(void) {
  g_final = 1;
  return MPI_SUCCESS;
}
int MPI_Finalized(int* flag) {
  *flag = g_final;
  return MPI_SUCCESS;
}
int MPI_Abort(MPI_Comm, int code) {
  exit(code);
  return MPI_SUCCESS;
}
int MPI_Comm_rank(MPI_Comm comm, int* rank) {
  *rank = 0;
  return pg::comm_valid(comm) ? MPI_SUCCESS : MPI_ERR_OTHER;
}
int MPI_Comm_size(MPI_Comm comm, int* size) {
  *size = 1;
  return pg::comm_valid(comm) ? MPI_SUCCESS : MPI_ERR_OTHER;
}
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm* nc) {
  if (!pg::comm_valid(comm)) return MPI_ERR_OTHER;
  *nc = new_handle(pg::comm_cart_dims(comm));
  return MPI_SUCCESS;
}
int MPI_Comm_free(MPI_Comm* comm) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (*comm >= 3 && (size_t)*comm < g_live.size()) g_live[*comm] = 0;
  *comm = MPI_COMM_NULL;
  return MPI_SUCCESS;
}
int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
int MPI_Allreduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
  if (s != MPI_IN_PLACE && s != r) memmove(r, s, (size_t)count * type_size(t));
  return MPI_SUCCESS;
}
int MPI_Reduce(const void* s, void* r, int count, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  if (s != MPI_IN_PLACE && s != r && r) memmove(r, s, (size_t)count * type_size(t));
  return MPI_SUCCESS;
}
int MPI_Cart_create(MPI_Comm comm, int ndims, const int* dims, const int*, int, MPI_Comm* cart) {
  if (!pg::comm_valid(comm) || ndims < 1) return MPI_ERR_OTHER;
  long p = 1;
  for (int t = 0; t < ndims; t++) p *= dims[t];
  if (p != 1) {
    *cart = MPI_COMM_NULL;
    return MPI_ERR_OTHER;
  }
  *cart = new_handle(ndims);
  return MPI_SUCCESS;
}
int MPI_Cartdim_get(MPI_Comm comm, int* ndims) {
  *ndims = pg::comm_cart_dims(comm);
  return MPI_SUCCESS;
}
int MPI_Cart_get(MPI_Comm comm, int maxdims, int* dims, int* periods, int* coords) {
  int nd = pg::comm_cart_dims(comm);
  for (int t = 0; t < maxdims && t < nd; t++) {
    dims[t] = 1;
    periods[t] = 1;
    coords[t] = 0;
  }
  return MPI_SUCCESS;
}
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int* coords) {
  int nd = pg::comm_cart_dims(comm);
  for (int t = 0; t < maxdims && t < nd; t++) coords[t] = 0;
  return rank == 0 ? MPI_SUCCESS : MPI_ERR_OTHER;
}
int MPI_Cart_rank(MPI_Comm, const int*, int* rank) {
  *rank = 0;
  return MPI_SUCCESS;
}
int MPI_Cart_shift(MPI_Comm, int, int, int* src, int* dst) {
  *src = 0;
  *dst = 0;
  return MPI_SUCCESS;
}
int MPI_Cart_sub(MPI_Comm comm, const int* remain, MPI_Comm* nc) {
  int nd = pg::comm_cart_dims(comm), k = 0;
  for (int t = 0; t < nd; t++) k += remain[t] ? 1 : 0;
  *nc = new_handle(k > 0 ? k : 1);
  return MPI_SUCCESS;
}
int MPI_Topo_test(MPI_Comm comm, int* status) {
  *status = pg::comm_cart_dims(comm) > 0 ? MPI_CART : MPI_UNDEFINED;
  return MPI_SUCCESS;
}
double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

}  // extern "C"
