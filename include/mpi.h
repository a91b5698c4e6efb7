/* Single-rank MPI stand-in for the GB300 build of the PFFT C API.
 *
 * The GB300 library runs every transform on one GPU, so the process mesh is
 * always 1 x 1 (x 1).  This header supplies just enough of MPI for PFFT user
 * code and PFFT-style test drivers to compile and run without an MPI
 * installation: one rank, Cartesian communicators of any rank whose
 * dimensions are all 1, reductions that copy, and a wall clock.
 *
 * Communicators are plain integer handles.  MPI_COMM_WORLD and MPI_COMM_SELF
 * are non-Cartesian; MPI_Cart_create returns a handle that remembers its
 * number of dimensions (PFFT derives the mesh rank from it).
 */
#ifndef PFFT_GB300_MPI_H
#define PFFT_GB300_MPI_H 1

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Group;
typedef int MPI_Request;
typedef struct {
  int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_COMM_NULL ((MPI_Comm)0)
#define MPI_COMM_WORLD ((MPI_Comm)1)
#define MPI_COMM_SELF ((MPI_Comm)2)

#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_UNDEFINED (-32766)
#define MPI_CART 1
#define MPI_GRAPH 2
#define MPI_PROC_NULL (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)2)
#define MPI_UNSIGNED ((MPI_Datatype)3)
#define MPI_LONG ((MPI_Datatype)4)
#define MPI_FLOAT ((MPI_Datatype)5)
#define MPI_DOUBLE ((MPI_Datatype)6)
#define MPI_LONG_DOUBLE ((MPI_Datatype)7)
#define MPI_LONG_LONG ((MPI_Datatype)8)
#define MPI_BYTE ((MPI_Datatype)9)

#define MPI_MAX ((MPI_Op)1)
#define MPI_MIN ((MPI_Op)2)
#define MPI_SUM ((MPI_Op)3)
#define MPI_PROD ((MPI_Op)4)

#define MPI_IN_PLACE ((void *)1)

int MPI_Init(int *argc, char ***argv);
int MPI_Initialized(int *flag);
int MPI_Finalize(void);
int MPI_Finalized(int *flag);
int MPI_Abort(MPI_Comm comm, int errorcode);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_dup(MPI_Comm comm, MPI_Comm *newcomm);
int MPI_Comm_free(MPI_Comm *comm);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Cart_create(MPI_Comm comm, int ndims, const int *dims, const int *periods, int reorder, MPI_Comm *comm_cart);
int MPI_Cartdim_get(MPI_Comm comm, int *ndims);
int MPI_Cart_get(MPI_Comm comm, int maxdims, int *dims, int *periods, int *coords);
int MPI_Cart_coords(MPI_Comm comm, int rank, int maxdims, int *coords);
int MPI_Cart_rank(MPI_Comm comm, const int *coords, int *rank);
int MPI_Cart_shift(MPI_Comm comm, int direction, int disp, int *rank_source, int *rank_dest);
int MPI_Cart_sub(MPI_Comm comm, const int *remain_dims, MPI_Comm *newcomm);
int MPI_Topo_test(MPI_Comm comm, int *status);
double MPI_Wtime(void);

#ifdef __cplusplus
}
#endif

#endif /* PFFT_GB300_MPI_H */
