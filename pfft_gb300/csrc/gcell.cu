// Ghost-cell exchange and reduce on one GPU.
//
// Reference: gcell/gcells_plan.c (plan_rgc_internal :80-199, local_size_gc
// :51-76, exchange_gc :379-398, reduce_gc :401-420, zero padding :424-455,
// truncation :458-486) and gcell/gcells_sendrecv.c.  With a single rank every
// neighbour is the rank itself, so the exchange is a periodic wrap of the
// compact block into the (gc_below + n + gc_above) box,
//     box[k] = block[(k - gc_below) mod n]   (per axis),
// and the reduce is its adjoint: every block cell receives the sum of all box
// cells that are its periodic images, then the box is truncated back to the
// compact block and the rest of the buffer is zeroed.
//
// Both operations are in place on the user's buffer, in one sweep over the
// data, as the reference pads in place from the back
// (pad_array_with_zeros_outside_3d, gcells_plan.c:424-455) before its halo
// messages:
//   exchange  1. k_gc_move (expand): every block row moves to its interior
//                position in the box, rows taken from the back in chunks;
//             2. k_gc_fill: every ghost cell copies its interior image.
//   reduce    1. k_gc_fold: every block cell with ghost images sums them,
//                in place at its interior position;
//             2. k_gc_move (compact): interior rows move back to the compact
//                block, chunks taken from the front; the rest is zeroed.
// A chunk's rows are staged in shared memory, so a chunk may overwrite its
// own source; a chunk writes only after every earlier chunk (taken by an
// atomic ticket, hence already running) whose source rows its writes cover
// has read them (per-chunk flags, bounded waits with an error word).  Rows
// longer than the staging area (more than 4096 doubles or 8192 floats) fall
// back to a copy of the data in plan scratch memory and a gather /
// scatter-add kernel.
#include <stdio.h>
#include <algorithm>
#include <string.h>
#include <chrono>
#include "../../include/pfft.h"
#include "../../include/pfft_gb300.h"
#include "core.h"

using namespace pg;

namespace {

struct GcDims {
  long long n[3], gb[3], ng[3];
  long long tuple;  // reals per cell
};

// box <- periodic wrap of the compact block held in src
template <class T>
__global__ void k_gc_gather(const T* __restrict__ src, T* __restrict__ box, GcDims g, long long ncell) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += stride) {
    long long r = c;
    long long k2 = r % g.ng[2];
    r /= g.ng[2];
    long long k1 = r % g.ng[1];
    long long k0 = r / g.ng[1];
    long long j0 = (k0 - g.gb[0]) % g.n[0];
    long long j1 = (k1 - g.gb[1]) % g.n[1];
    long long j2 = (k2 - g.gb[2]) % g.n[2];
    if (j0 < 0) j0 += g.n[0];
    if (j1 < 0) j1 += g.n[1];
    if (j2 < 0) j2 += g.n[2];
    const T* s = src + ((j0 * g.n[1] + j1) * g.n[2] + j2) * g.tuple;
    T* d = box + c * g.tuple;
    for (long long h = 0; h < g.tuple; h++) d[h] = s[h];
  }
}

// block cell j <- sum of its periodic images in the box held in src
template <class T>
__global__ void k_gc_reduce(const T* __restrict__ src, T* __restrict__ blk, GcDims g, long long ncell) {
  long long stride = (long long)gridDim.x * blockDim.x;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += stride) {
    long long r = c;
    long long j2 = r % g.n[2];
    r /= g.n[2];
    long long j1 = r % g.n[1];
    long long j0 = r / g.n[1];
    // first image along each axis
    long long s0 = j0 + g.gb[0], s1 = j1 + g.gb[1], s2 = j2 + g.gb[2];
    s0 -= (s0 / g.n[0]) * g.n[0];
    s1 -= (s1 / g.n[1]) * g.n[1];
    s2 -= (s2 / g.n[2]) * g.n[2];
    for (long long h = 0; h < g.tuple; h++) {
      T acc = 0;
      for (long long k0 = s0; k0 < g.ng[0]; k0 += g.n[0])
        for (long long k1 = s1; k1 < g.ng[1]; k1 += g.n[1])
          for (long long k2 = s2; k2 < g.ng[2]; k2 += g.n[2])
            acc += src[((k0 * g.ng[1] + k1) * g.ng[2] + k2) * g.tuple + h];
      blk[c * g.tuple + h] = acc;
    }
  }
}

// ---- single-sweep in-place kernels ------------------------------------------------
constexpr int GC_THREADS = 256;
constexpr int GC_STAGE_BYTES = 32 * 1024;  // staging area of a chunk (static shared memory)
constexpr int GC_MAX_ROWS = 1024;          // rows per chunk (row-start table)

struct GcMove {
  long long rows;        // block rows (n0 * n1)
  long long n1;          // block extent of axis 1
  long long RS, RB;      // scalars per block row (n2 * tuple) and per box row (ng2 * tuple)
  long long gb0, gb1, ng1;
  long long off2;        // gc_below[2] * tuple: start of the interior in a box row
  long long R;           // rows per chunk
  long long nchunks;
  unsigned* ticket;
  unsigned* flags;       // one per chunk: the epoch once the chunk's rows are read
  int* err;
  unsigned epoch;
  unsigned rs_magic;     // 0xFFFFFFFF / RS + 1 (RS > 1): f / RS = umulhi(f, rs_magic) for f, RS < 2^16
  unsigned rsv_magic;    // the same for RSV = RS / W, the 16-byte vectors of a block row (vector path)
  long long spin_limit;
};

// Vector path of the move: every row start, row length and the buffer 16-byte
// aligned; each thread then moves its share of a chunk (GC_STAGE_BYTES / 16 /
// GC_THREADS = 8 vectors) as 16-byte vectors, four loads issued before their
// stores, instead of one 8-byte access at a time.
constexpr int GC_VPT = GC_STAGE_BYTES / 16 / GC_THREADS;

__device__ __forceinline__ long long gc_box_start(const GcMove& m, long long row) {
  const long long j0 = row / m.n1, j1 = row - j0 * m.n1;
  return ((j0 + m.gb0) * m.ng1 + j1 + m.gb1) * m.RB + m.off2;
}

// EXPAND: block rows -> interior box rows, chunks from the back; otherwise
// interior box rows -> block rows, chunks from the front
// chunk's rows <-> stage as 16-byte vectors (VEC path): contiguous block
// rows on one side, box rows (start boxrow[q], RSV vectors) on the other;
// four vectors in flight per thread, twice
template <class T, bool TO_STAGE, bool BOX>
__device__ __forceinline__ void gc_vec_move(T* __restrict__ data, uint4* stv, const long long* boxrow, long long blk0,
                                            unsigned nv, const GcMove& m) {
  constexpr int W = 16 / (int)sizeof(T);
  constexpr int K = 4;
  const unsigned RSV = (unsigned)(m.RS / W);
#pragma unroll 1
  for (int k0 = 0; k0 < GC_VPT; k0 += K) {
    uint4 tmp[K];
#pragma unroll
    for (int k = 0; k < K; k++) {
      const unsigned f = threadIdx.x + (k0 + k) * GC_THREADS;
      if (f >= nv) continue;
      if (TO_STAGE) {
        if (BOX) {
          const unsigned q = RSV == 1 ? f : __umulhi(f, m.rsv_magic);
          tmp[k] = ((const uint4*)data)[boxrow[q] / W + (f - q * RSV)];
        } else {
          tmp[k] = ((const uint4*)data)[blk0 / W + f];
        }
      } else {
        tmp[k] = stv[f];
      }
    }
#pragma unroll
    for (int k = 0; k < K; k++) {
      const unsigned f = threadIdx.x + (k0 + k) * GC_THREADS;
      if (f >= nv) continue;
      if (TO_STAGE) {
        stv[f] = tmp[k];
      } else if (BOX) {
        const unsigned q = RSV == 1 ? f : __umulhi(f, m.rsv_magic);
        ((uint4*)data)[boxrow[q] / W + (f - q * RSV)] = tmp[k];
      } else {
        ((uint4*)data)[blk0 / W + f] = tmp[k];
      }
    }
  }
}

template <class T, bool EXPAND, bool VEC>
__global__ void __launch_bounds__(GC_THREADS, VEC ? 4 : 1) k_gc_move(T* __restrict__ data, const GcMove m) {
  __shared__ __align__(16) unsigned char stage_raw[GC_STAGE_BYTES];
  __shared__ long long boxrow[GC_MAX_ROWS];
  __shared__ long long s_chunk;
  T* stage = (T*)stage_raw;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) s_chunk = (long long)atomicAdd(m.ticket, 1u);
    __syncthreads();
    const long long c = s_chunk;
    if (c >= m.nchunks) break;
    long long r_lo, r_hi;
    if (EXPAND) {
      r_hi = m.rows - c * m.R;
      r_lo = r_hi - m.R > 0 ? r_hi - m.R : 0;
    } else {
      r_lo = c * m.R;
      r_hi = r_lo + m.R < m.rows ? r_lo + m.R : m.rows;
    }
    const int nr = (int)(r_hi - r_lo);
    for (int q = tid; q < nr; q += GC_THREADS) boxrow[q] = gc_box_start(m, r_lo + q);
    __syncthreads();
    const unsigned nsc = (unsigned)(nr * m.RS);
    // read the chunk's rows
    if (VEC) {
      gc_vec_move<T, true, !EXPAND>(data, (uint4*)stage_raw, boxrow, r_lo * m.RS, nsc / (16 / sizeof(T)), m);
    } else if (EXPAND) {
      const T* src = data + r_lo * m.RS;  // block rows are contiguous
      for (unsigned f = tid; f < nsc; f += GC_THREADS) stage[f] = src[f];
    } else {
      for (unsigned f = tid; f < nsc; f += GC_THREADS) {
        const unsigned q = m.RS == 1 ? f : __umulhi(f, m.rs_magic);
        stage[f] = data[boxrow[q] + (f - q * (unsigned)m.RS)];
      }
    }
    __syncthreads();
    if (tid == 0) {
      __threadfence();
      atomicExch(m.flags + c, m.epoch);
    }
    // earlier chunks whose source rows this chunk's writes cover
    long long w_lo = c, w_hi = c - 1;
    if (EXPAND) {
      const long long whi = boxrow[nr - 1] + m.RS - 1;  // last scalar written
      long long rmax = whi / m.RS;
      if (rmax > m.rows - 1) rmax = m.rows - 1;
      if (rmax >= r_hi) w_lo = (m.rows - 1 - rmax) / m.R;
    } else if (r_lo > 0) {
      // first row whose box source ends past this chunk's first written scalar
      const long long wlo = r_lo * m.RS;
      long long a = 0, b = r_lo;
      while (a < b) {
        const long long mid = (a + b) / 2;
        if (gc_box_start(m, mid) + m.RS > wlo)
          b = mid;
        else
          a = mid + 1;
      }
      if (a < r_lo) w_lo = a / m.R;
    }
    for (long long q = w_lo + tid; q <= w_hi; q += GC_THREADS) {
      const volatile unsigned* fl = m.flags + q;
      long long it = 0;
      while (*fl != m.epoch) {
        if (++it > m.spin_limit) {
          atomicExch(m.err, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    __syncthreads();
    // write
    if (VEC) {
      gc_vec_move<T, false, EXPAND>(data, (uint4*)stage_raw, boxrow, r_lo * m.RS, nsc / (16 / sizeof(T)), m);
    } else if (EXPAND) {
      for (unsigned f = tid; f < nsc; f += GC_THREADS) {
        const unsigned q = m.RS == 1 ? f : __umulhi(f, m.rs_magic);
        data[boxrow[q] + (f - q * (unsigned)m.RS)] = stage[f];
      }
    } else {
      T* dst = data + r_lo * m.RS;
      for (unsigned f = tid; f < nsc; f += GC_THREADS) dst[f] = stage[f];
    }
    __syncthreads();
  }
}

// k mod n in [0, n); one compare for the usual |k| < 2n
__device__ __forceinline__ long long gc_wrap(long long k, long long n) {
  if (k >= 0 && k < n) return k;
  if (k < 0 && k >= -n) return k + n;
  if (k >= n && k < 2 * n) return k - n;
  const long long j = k % n;
  return j < 0 ? j + n : j;
}

// Work lists of the fill and the fold (host-computed counts).  Part A: rows
// of which only a few cells along axis 2 take part (per scalars each), rpw
// rows to a warp, a lane to a scalar; part B: rows of which every cell takes
// part, a warp to a row.  Row-internal indexes are 32-bit: a row of the
// single-sweep path holds at most 8192 scalars.
struct GcWork {
  long long rowsA, rowsB;
  int per, rpw;
};

// every ghost cell of the box <- its interior image.  Part A: the ghost cells
// at both ends of every interior row (k0, k1 inside the block); part B: the
// ghost rows (k0 or k1 outside), enumerated as the ghost planes along axis 0
// and then the ghost rows of the interior planes.  Both read interior cells
// only, which neither writes.
template <class T>
__global__ void __launch_bounds__(GC_THREADS) k_gc_fill(T* __restrict__ data, GcDims g, GcWork w) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (GC_THREADS / 32);
  const long long n0 = g.n[0], n1 = g.n[1], n2 = g.n[2], gb0 = g.gb[0], gb1 = g.gb[1], gb2 = g.gb[2];
  const long long ng1 = g.ng[1], e0 = g.ng[0] - n0, e1 = ng1 - n1;
  const unsigned tu = (unsigned)g.tuple, RB = (unsigned)(g.ng[2] * g.tuple);
  const long long groupsA = (w.rowsA + w.rpw - 1) / w.rpw;
  const int lr = w.rpw > 1 ? lane / w.per : 0, lc0 = w.rpw > 1 ? lane % w.per : lane;
  for (long long q = (long long)blockIdx.x * (GC_THREADS / 32) + (threadIdx.x >> 5); q < groupsA + w.rowsB; q += warps) {
    if (q < groupsA) {
      const long long row = q * w.rpw + lr;
      if (lr >= w.rpw || row >= w.rowsA) continue;
      const long long j0 = row / n1, j1 = row - j0 * n1;
      T* base = data + ((j0 + gb0) * ng1 + j1 + gb1) * RB;
      for (int lc = lc0; lc < w.per; lc += 32) {
        const unsigned c = (unsigned)lc / tu, h = (unsigned)lc - c * tu;
        const long long k2 = c < gb2 ? c : c + n2;
        base[k2 * tu + h] = base[(gc_wrap(k2 - gb2, n2) + gb2) * tu + h];
      }
    } else {
      const long long r = q - groupsA, planes = e0 * ng1;
      long long k0, k1;
      if (r < planes) {
        const long long p = r / ng1;
        k1 = r - p * ng1;
        k0 = p < gb0 ? p : p + n0;
      } else {
        const long long p = (r - planes) / e1, c = r - planes - p * e1;
        k0 = gb0 + p;
        k1 = c < gb1 ? c : c + n1;
      }
      const T* src = data + ((gc_wrap(k0 - gb0, n0) + gb0) * ng1 + gc_wrap(k1 - gb1, n1) + gb1) * RB;
      T* dst = data + (k0 * ng1 + k1) * RB;
      for (unsigned t = lane; t < RB; t += 32) {
        const unsigned k2 = t / tu, h = t - k2 * tu;
        dst[t] = src[(gc_wrap((long long)k2 - gb2, n2) + gb2) * tu + h];
      }
    }
  }
}

// every block cell with more than one image <- the sum of its images (k0,
// k1, k2 ascending), written at its interior position.  A cell j has the
// images s, s + n, ... below ng per axis, s = (j + gb) mod n: more than one
// for s < m = min(ng - n, n).  Part A: the rows with one image along axes 0
// and 1 (s0 >= m0, s1 >= m1; then k0 = s0, k1 = s1 is the interior row),
// their cells s2 < m2; part B: the rows with s0 < m0 or s1 < m1, all cells.
// A thread reads only its own cell's images, so the in-place sums do not
// race.
template <class T>
__global__ void __launch_bounds__(GC_THREADS) k_gc_fold(T* __restrict__ data, GcDims g, GcWork w) {
  const int lane = threadIdx.x & 31;
  const long long warps = (long long)gridDim.x * (GC_THREADS / 32);
  const long long n0 = g.n[0], n1 = g.n[1], n2 = g.n[2], gb0 = g.gb[0], gb1 = g.gb[1], gb2 = g.gb[2];
  const long long ng0 = g.ng[0], ng1 = g.ng[1], ng2 = g.ng[2];
  const long long m0 = ng0 - n0 < n0 ? ng0 - n0 : n0, m1 = ng1 - n1 < n1 ? ng1 - n1 : n1;
  const unsigned tu = (unsigned)g.tuple, RB = (unsigned)(ng2 * g.tuple);
  const long long groupsA = (w.rowsA + w.rpw - 1) / w.rpw;
  const int lr = w.rpw > 1 ? lane / w.per : 0, lc0 = w.rpw > 1 ? lane % w.per : lane;
  for (long long q = (long long)blockIdx.x * (GC_THREADS / 32) + (threadIdx.x >> 5); q < groupsA + w.rowsB; q += warps) {
    if (q < groupsA) {
      const long long row = q * w.rpw + lr;
      if (lr >= w.rpw || row >= w.rowsA) continue;
      const long long a0 = row / (n1 - m1);
      T* rowp = data + ((m0 + a0) * ng1 + m1 + row - a0 * (n1 - m1)) * RB;
      for (int lc = lc0; lc < w.per; lc += 32) {
        const unsigned s2 = (unsigned)lc / tu, h = (unsigned)lc - s2 * tu;
        T acc = 0;
        for (long long k2 = s2; k2 < ng2; k2 += n2) acc += rowp[k2 * tu + h];
        rowp[(gc_wrap(s2 - gb2, n2) + gb2) * tu + h] = acc;
      }
    } else {
      const long long r = q - groupsA;
      long long s0, s1;
      if (r < m0 * n1) {
        s0 = r / n1;
        s1 = gc_wrap(r - s0 * n1 + gb1, n1);
      } else {
        const long long p = (r - m0 * n1) / m1;
        s0 = m0 + p;
        s1 = r - m0 * n1 - p * m1;
      }
      T* at = data + ((gc_wrap(s0 - gb0, n0) + gb0) * ng1 + gc_wrap(s1 - gb1, n1) + gb1) * RB;
      for (unsigned t = lane; t < (unsigned)(n2 * tu); t += 32) {
        const unsigned j2 = t / tu, h = t - j2 * tu;
        const long long s2 = gc_wrap(j2 + gb2, n2);
        T acc = 0;
        for (long long k0 = s0; k0 < ng0; k0 += n0)
          for (long long k1 = s1; k1 < ng1; k1 += n1)
            for (long long k2 = s2; k2 < ng2; k2 += n2) acc += data[((k0 * ng1 + k1) * ng2 + k2) * tu + h];
        at[(j2 + gb2) * tu + h] = acc;
      }
    }
  }
}

// fill: part A the interior rows' end cells, part B the ghost rows
GcWork gc_fill_work(const GcDims& g) {
  GcWork w;
  const long long e2 = g.ng[2] - g.n[2];
  w.per = (int)(e2 * g.tuple);
  w.rowsA = w.per > 0 ? g.n[0] * g.n[1] : 0;
  w.rowsB = (g.ng[0] - g.n[0]) * g.ng[1] + g.n[0] * (g.ng[1] - g.n[1]);
  w.rpw = w.per > 0 && w.per <= 16 ? 32 / w.per : 1;
  if (w.per == 0) w.per = 1;
  return w;
}
// fold: part A the single-image rows' cells s2 < m2, part B the other rows
GcWork gc_fold_work(const GcDims& g) {
  GcWork w;
  const long long m0 = std::min(g.ng[0] - g.n[0], g.n[0]), m1 = std::min(g.ng[1] - g.n[1], g.n[1]);
  const long long m2 = std::min(g.ng[2] - g.n[2], g.n[2]);
  w.per = (int)(m2 * g.tuple);
  w.rowsA = w.per > 0 ? (g.n[0] - m0) * (g.n[1] - m1) : 0;
  w.rowsB = m0 * g.n[1] + (g.n[0] - m0) * m1;
  w.rpw = w.per > 0 && w.per <= 16 ? 32 / w.per : 1;
  if (w.per == 0) w.per = 1;
  return w;
}

struct GcPlan {
  int prec;  // 0 float, 1 double
  void* data;
  GcDims g;
  long long ncomp, nbox;  // cells
  void* scratch = nullptr;  // only rows longer than the staging area (copy + gather path)
  size_t scratch_bytes = 0;
  bool single_sweep = true;
  long long R = 1, nchunks = 0;  // rows per chunk, chunks of the in-place moves
  unsigned* ctl = nullptr;       // device: ticket, error word, one flag per chunk
  int* h_err = nullptr;          // pinned copy of the error word
  unsigned epoch = 0;
  int sms = 1;
  cudaStream_t stream = 0;
  // timers (gcell/gctimer.c layout: iter, whole, pad_zeros, exchange)
  double texg[4] = {0, 0, 0, 0};
  double tred[4] = {0, 0, 0, 0};
};

size_t esz(const GcPlan* p) { return p->prec ? sizeof(double) : sizeof(float); }

int launch_grid(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 32) b = 152 * 32;
  return (int)(b < 1 ? 1 : b);
}

bool dev_ptr(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

void gc_free(GcPlan* p) {
  if (!p) return;
  if (p->scratch) cudaFree(p->scratch);
  if (p->ctl) cudaFree(p->ctl);
  if (p->h_err) cudaFreeHost(p->h_err);
  delete p;
}

GcPlan* make_gc(int prec, int rnk, const INT* n_user, INT howmany, const INT* gcb_user, const INT* gca_user,
                void* data, MPI_Comm comm, unsigned flags, bool complex_data) {
  INT n[8], gcb[8], gca[8];
  for (int t = 0; t < rnk; t++) {
    n[t] = n_user[t];
    gcb[t] = gcb_user ? gcb_user[t] : 0;
    gca[t] = gca_user ? gca_user[t] : 0;
  }
  INT tuple = howmany;
  if (complex_data) {  // api/api-adv.c:295-324
    flags &= ~GC_PADDED;
    if (flags & GC_R2C) {
      n[rnk - 1] = n[rnk - 1] / 2 + 1;
      flags &= ~GC_R2C;
    }
    tuple = 2 * howmany;
  }
  if (flags & GC_PADDED) n[rnk - 1] = 2 * (n[rnk - 1] / 2 + 1);  // api/api-adv.c:250-252
  bool nothing = true;
  for (int t = 0; t < rnk; t++)
    if (gcb[t] != 0 || gca[t] != 0) nothing = false;
  if (nothing) return nullptr;
  if (rnk != 3) {
    fprintf(stderr, "Error: Gcell send only available for three dimensions.\n");
    return nullptr;
  }
  if (!comm_valid(comm)) return nullptr;
  int cd = comm_cart_dims(comm);
  int rnk_pm = cd > 0 ? cd : 1;
  // gcell/gcells_plan.c:222-234: cyclic shift of the distributed dims
  INT pn[3], pgb[3], pga[3];
  for (int t = 0; t < 3; t++) {
    int s = (t < rnk_pm && (flags & GC_TRANSPOSED)) ? (t + 1) % rnk_pm : t;
    pn[t] = n[s];
    pgb[t] = gcb[s];
    pga[t] = gca[s];
  }
  GcPlan* p = new GcPlan();
  p->prec = prec;
  p->data = data;
  p->ncomp = 1;
  p->nbox = 1;
  for (int t = 0; t < 3; t++) {
    if (pn[t] <= 0 || pgb[t] < 0 || pga[t] < 0) {
      gc_free(p);
      return nullptr;
    }
    p->g.n[t] = pn[t];
    p->g.gb[t] = pgb[t];
    p->g.ng[t] = pgb[t] + pn[t] + pga[t];
    p->ncomp *= pn[t];
    p->nbox *= p->g.ng[t];
  }
  p->g.tuple = tuple;
  const long long RS = p->g.n[2] * tuple;
  const long long cap = GC_STAGE_BYTES / (long long)esz(p);
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, dev);
  if (p->sms < 1) p->sms = 1;
  if (RS <= cap) {
    p->R = std::min<long long>(GC_MAX_ROWS, cap / RS);
    const long long rows = p->g.n[0] * p->g.n[1];
    p->nchunks = (rows + p->R - 1) / p->R;
    if (cuda_check(cudaMalloc(&p->ctl, sizeof(unsigned) * (size_t)(2 + p->nchunks)), "ghost-cell flags") ||
        cuda_check(cudaMemset(p->ctl, 0, sizeof(unsigned) * (size_t)(2 + p->nchunks)), "ghost-cell flags") ||
        cuda_check(cudaMallocHost(&p->h_err, sizeof(int)), "ghost-cell error word")) {
      gc_free(p);
      return nullptr;
    }
  } else {
    p->single_sweep = false;
    p->scratch_bytes = (size_t)p->nbox * tuple * esz(p);
    if (cuda_check(cudaMalloc(&p->scratch, p->scratch_bytes), "ghost-cell scratch")) {
      gc_free(p);
      return nullptr;
    }
  }
  return p;
}

GcMove gc_move_args(GcPlan* p) {
  GcMove m;
  m.rows = p->g.n[0] * p->g.n[1];
  m.n1 = p->g.n[1];
  m.RS = p->g.n[2] * p->g.tuple;
  m.RB = p->g.ng[2] * p->g.tuple;
  m.gb0 = p->g.gb[0];
  m.gb1 = p->g.gb[1];
  m.ng1 = p->g.ng[1];
  m.off2 = p->g.gb[2] * p->g.tuple;
  m.R = p->R;
  m.nchunks = p->nchunks;
  m.ticket = p->ctl;
  m.err = (int*)(p->ctl + 1);
  m.flags = p->ctl + 2;
  if (++p->epoch == 0) p->epoch = 1;  // flags start at 0, so epoch 0 is never used
  m.epoch = p->epoch;
  m.rs_magic = m.RS > 1 ? (unsigned)(0xFFFFFFFFull / (unsigned long long)m.RS + 1) : 0u;
  const long long W = 16 / esz(p), RSV = m.RS / W;
  m.rsv_magic = RSV > 1 ? (unsigned)(0xFFFFFFFFull / (unsigned long long)RSV + 1) : 0u;
  m.spin_limit = 20000000;  // about 2 s of 64 ns naps
  return m;
}

template <class T, bool EXPAND>
int gc_move(GcPlan* p, void* data) {
  cudaError_t e = cudaMemsetAsync(p->ctl, 0, 2 * sizeof(unsigned), p->stream);  // ticket, error word
  if (e != cudaSuccess) return (int)e;
  const GcMove m = gc_move_args(p);
  const long long grid = std::min<long long>(m.nchunks, (long long)p->sms * 4);
  // 16-byte vectors when every row start and length is a multiple of 16 bytes
  const long long W = 16 / (long long)sizeof(T);
  const bool vec = ((uintptr_t)data & 15) == 0 && m.RS % W == 0 && m.RB % W == 0 && m.off2 % W == 0;
  if (grid > 0 && vec) k_gc_move<T, EXPAND, true><<<(unsigned)grid, GC_THREADS, 0, p->stream>>>((T*)data, m);
  if (grid > 0 && !vec) k_gc_move<T, EXPAND, false><<<(unsigned)grid, GC_THREADS, 0, p->stream>>>((T*)data, m);
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  return (int)cudaMemcpyAsync(p->h_err, p->ctl + 1, sizeof(int), cudaMemcpyDeviceToHost, p->stream);
}

int gc_rows_grid(const GcPlan* p, long long rows) {
  const long long want = (rows + (GC_THREADS / 32) - 1) / (GC_THREADS / 32);
  return (int)std::max(1LL, std::min<long long>(want, (long long)p->sms * 8));
}

template <class T>
int gc_exchange_t(GcPlan* p, void* data) {
  if (!p->single_sweep) {
    size_t cb = (size_t)p->ncomp * p->g.tuple * sizeof(T);
    cudaError_t e = cudaMemcpyAsync(p->scratch, data, cb, cudaMemcpyDeviceToDevice, p->stream);
    if (e != cudaSuccess) return (int)e;
    k_gc_gather<T><<<launch_grid(p->nbox), 256, 0, p->stream>>>((const T*)p->scratch, (T*)data, p->g, p->nbox);
    return (int)cudaGetLastError();
  }
  int rc = gc_move<T, true>(p, data);
  if (rc) return rc;
  const GcWork w = gc_fill_work(p->g);
  const long long units = (w.rowsA + w.rpw - 1) / w.rpw + w.rowsB;
  if (units > 0) k_gc_fill<T><<<gc_rows_grid(p, units), GC_THREADS, 0, p->stream>>>((T*)data, p->g, w);
  return (int)cudaGetLastError();
}

template <class T>
int gc_reduce_t(GcPlan* p, void* data) {
  size_t bb = (size_t)p->nbox * p->g.tuple * sizeof(T);
  size_t cb = (size_t)p->ncomp * p->g.tuple * sizeof(T);
  cudaError_t e;
  if (!p->single_sweep) {
    e = cudaMemcpyAsync(p->scratch, data, bb, cudaMemcpyDeviceToDevice, p->stream);
    if (e != cudaSuccess) return (int)e;
    k_gc_reduce<T><<<launch_grid(p->ncomp), 256, 0, p->stream>>>((const T*)p->scratch, (T*)data, p->g, p->ncomp);
  } else {
    const GcWork w = gc_fold_work(p->g);
    const long long units = (w.rowsA + w.rpw - 1) / w.rpw + w.rowsB;
    if (units > 0) k_gc_fold<T><<<gc_rows_grid(p, units), GC_THREADS, 0, p->stream>>>((T*)data, p->g, w);
    e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
    int rc = gc_move<T, false>(p, data);
    if (rc) return rc;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return (int)e;
  if (bb > cb) e = cudaMemsetAsync((char*)data + cb, 0, bb - cb, p->stream);
  return (int)e;
}

void gc_run(GcPlan* p, bool reduce) {
  if (!p) return;
  auto t0 = std::chrono::steady_clock::now();
  size_t bb = (size_t)p->nbox * p->g.tuple * esz(p);
  void* d = p->data;
  void* tmp = nullptr;
  if (!dev_ptr(d)) {  // host buffer: stage through a device copy
    if (cuda_check(cudaMalloc(&tmp, bb), "ghost-cell staging")) return;
    size_t in_b = reduce ? bb : (size_t)p->ncomp * p->g.tuple * esz(p);
    if (cuda_check(cudaMemcpyAsync(tmp, d, in_b, cudaMemcpyHostToDevice, p->stream), "ghost-cell upload")) {
      cudaFree(tmp);
      return;
    }
    d = tmp;
  }
  int rc;
  if (reduce)
    rc = p->prec ? gc_reduce_t<double>(p, d) : gc_reduce_t<float>(p, d);
  else
    rc = p->prec ? gc_exchange_t<double>(p, d) : gc_exchange_t<float>(p, d);
  if (!rc && tmp) rc = (int)cudaMemcpyAsync(p->data, tmp, bb, cudaMemcpyDeviceToHost, p->stream);
  if (!rc) rc = (int)cudaStreamSynchronize(p->stream);
  if (tmp) cudaFree(tmp);
  if (rc) {
    cuda_check((cudaError_t)rc, reduce ? "reduce" : "exchange");
    return;
  }
  if (p->single_sweep && *p->h_err) {
    report("%s: a chunk's wait for the rows it overwrites timed out; the result is not valid",
           reduce ? "reduce" : "exchange");
    return;
  }
  double dt = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  double* tm = reduce ? p->tred : p->texg;
  tm[0] += 1;
  tm[1] += dt;
  tm[3] += dt;
}

struct GcTimer {
  double v[4];
};

}  // namespace

struct pfft_gcplan_s {
  GcPlan* p;
};
struct pfftf_gcplan_s {
  GcPlan* p;
};
struct pfft_gctimer_s {
  GcTimer t;
};
struct pfftf_gctimer_s {
  GcTimer t;
};

#define PG_GC_API(PX, PREC, R, C)                                                                          \
  extern "C" {                                                                                             \
  INT PX##local_size_many_gc(int rnk, const INT* ln, const INT* ls, INT howmany, const INT* gcb,          \
                             const INT* gca, INT* lngc, INT* lgcs) {                                      \
    INT mem = howmany;                                                                                     \
    for (int t = 0; t < rnk; t++) {                                                                        \
      INT b = gcb ? gcb[t] : 0, a = gca ? gca[t] : 0;                                                      \
      lngc[t] = b + ln[t] + a;                                                                             \
      lgcs[t] = ls[t] - b;                                                                                 \
      mem *= lngc[t];                                                                                      \
    }                                                                                                      \
    return mem;                                                                                            \
  }                                                                                                        \
  INT PX##local_size_gc(int rnk, const INT* ln, const INT* ls, const INT* gcb, const INT* gca, INT* lngc,  \
                        INT* lgcs) {                                                                       \
    return PX##local_size_many_gc(rnk, ln, ls, 1, gcb, gca, lngc, lgcs);                                   \
  }                                                                                                        \
  INT PX##local_size_gc_3d(const INT* ln, const INT* ls, const INT* gcb, const INT* gca, INT* lngc,        \
                           INT* lgcs) {                                                                    \
    return PX##local_size_many_gc(3, ln, ls, 1, gcb, gca, lngc, lgcs);                                     \
  }                                                                                                        \
  static PX##gcplan PX##gcwrap(GcPlan* p) {                                                                \
    if (!p) return nullptr;                                                                                \
    PX##gcplan w = new PX##gcplan_s;                                                                       \
    w->p = p;                                                                                              \
    return w;                                                                                              \
  }                                                                                                        \
  PX##gcplan PX##plan_many_rgc(int rnk, const INT* n, INT hm, const INT*, const INT* gcb, const INT* gca,  \
                               R* data, MPI_Comm comm, unsigned fl) {                                     \
    return PX##gcwrap(make_gc(PREC, rnk, n, hm, gcb, gca, data, comm, fl, false));                         \
  }                                                                                                        \
  PX##gcplan PX##plan_many_cgc(int rnk, const INT* n, INT hm, const INT*, const INT* gcb, const INT* gca,  \
                               C* data, MPI_Comm comm, unsigned fl) {                                     \
    return PX##gcwrap(make_gc(PREC, rnk, n, hm, gcb, gca, data, comm, fl, true));                          \
  }                                                                                                        \
  PX##gcplan PX##plan_rgc(int rnk, const INT* n, const INT* gcb, const INT* gca, R* data, MPI_Comm comm,   \
                          unsigned fl) {                                                                  \
    return PX##plan_many_rgc(rnk, n, 1, nullptr, gcb, gca, data, comm, fl);                                \
  }                                                                                                        \
  PX##gcplan PX##plan_cgc(int rnk, const INT* n, const INT* gcb, const INT* gca, C* data, MPI_Comm comm,   \
                          unsigned fl) {                                                                  \
    return PX##plan_many_cgc(rnk, n, 1, nullptr, gcb, gca, data, comm, fl);                                \
  }                                                                                                        \
  PX##gcplan PX##plan_rgc_3d(const INT* n, const INT* gcb, const INT* gca, R* data, MPI_Comm comm,         \
                             unsigned fl) {                                                               \
    return PX##plan_rgc(3, n, gcb, gca, data, comm, fl);                                                   \
  }                                                                                                        \
  PX##gcplan PX##plan_cgc_3d(const INT* n, const INT* gcb, const INT* gca, C* data, MPI_Comm comm,         \
                             unsigned fl) {                                                               \
    return PX##plan_cgc(3, n, gcb, gca, data, comm, fl);                                                   \
  }                                                                                                        \
  void PX##exchange(PX##gcplan ths) {                                                                      \
    if (ths) gc_run(ths->p, false);                                                                        \
  }                                                                                                        \
  void PX##reduce(PX##gcplan ths) {                                                                        \
    if (ths) gc_run(ths->p, true);                                                                         \
  }                                                                                                        \
  void PX##destroy_gcplan(PX##gcplan ths) {                                                                \
    if (!ths) return;                                                                                      \
    gc_free(ths->p);                                                                                       \
    delete ths;                                                                                            \
  }                                                                                                        \
  int PX##gb300_gc_set_stream(PX##gcplan ths, void* stream) {                                              \
    if (!ths) return -1;                                                                                   \
    ths->p->stream = (cudaStream_t)stream;                                                                 \
    return 0;                                                                                              \
  }                                                                                                        \
  void PX##reset_gctimers(PX##gcplan ths) {                                                                \
    if (!ths) return;                                                                                      \
    memset(ths->p->texg, 0, sizeof(ths->p->texg));                                                         \
    memset(ths->p->tred, 0, sizeof(ths->p->tred));                                                         \
  }                                                                                                        \
  PX##gctimer PX##get_gctimer_exg(const PX##gcplan ths) {                                                  \
    PX##gctimer t = new PX##gctimer_s;                                                                     \
    memcpy(t->t.v, ths->p->texg, sizeof(t->t.v));                                                          \
    return t;                                                                                              \
  }                                                                                                        \
  PX##gctimer PX##get_gctimer_red(const PX##gcplan ths) {                                                  \
    PX##gctimer t = new PX##gctimer_s;                                                                     \
    memcpy(t->t.v, ths->p->tred, sizeof(t->t.v));                                                          \
    return t;                                                                                              \
  }                                                                                                        \
  static void PX##fprint_gct(FILE* f, const char* pre, const double* v) {                                  \
    double it = v[0] > 0 ? v[0] : 1;                                                                       \
    fprintf(f, "%s(1) = %.6e;  %% whole\n", pre, v[1] / it);                                               \
    fprintf(f, "%s_pad_zeros(1) = %.6e;\n%s_exchange(1) = %.6e;\n", pre, v[2] / it, pre, v[3] / it);       \
  }                                                                                                        \
  void PX##print_average_gctimer(const PX##gcplan ths, MPI_Comm) {                                         \
    PX##fprint_gct(stdout, "pfft_gc_exg", ths->p->texg);                                                   \
    PX##fprint_gct(stdout, "pfft_gc_red", ths->p->tred);                                                   \
  }                                                                                                        \
  void PX##print_average_gctimer_adv(const PX##gcplan ths, MPI_Comm c) { PX##print_average_gctimer(ths, c); } \
  void PX##write_average_gctimer(const PX##gcplan ths, const char* name, MPI_Comm) {                       \
    FILE* f = fopen(name, "a");                                                                            \
    if (!f) return;                                                                                        \
    PX##fprint_gct(f, "pfft_gc_exg", ths->p->texg);                                                        \
    PX##fprint_gct(f, "pfft_gc_red", ths->p->tred);                                                        \
    fclose(f);                                                                                             \
  }                                                                                                        \
  void PX##write_average_gctimer_adv(const PX##gcplan ths, const char* name, MPI_Comm c) {                 \
    PX##write_average_gctimer(ths, name, c);                                                               \
  }                                                                                                        \
  PX##gctimer PX##copy_gctimer(const PX##gctimer o) {                                                      \
    PX##gctimer t = new PX##gctimer_s;                                                                     \
    t->t = o->t;                                                                                           \
    return t;                                                                                              \
  }                                                                                                        \
  void PX##average_gctimer(PX##gctimer t) {                                                                \
    if (t->t.v[0] <= 0) return;                                                                            \
    for (int k = 1; k < 4; k++) t->t.v[k] /= t->t.v[0];                                                    \
    t->t.v[0] = 1;                                                                                         \
  }                                                                                                        \
  PX##gctimer PX##add_gctimers(const PX##gctimer a, const PX##gctimer b) {                                 \
    PX##gctimer t = new PX##gctimer_s;                                                                     \
    for (int k = 0; k < 4; k++) t->t.v[k] = a->t.v[k] + b->t.v[k];                                         \
    return t;                                                                                              \
  }                                                                                                        \
  PX##gctimer PX##reduce_max_gctimer(const PX##gctimer t, MPI_Comm) { return PX##copy_gctimer(t); }        \
  void PX##convert_gctimer2vec(const PX##gctimer t, double* v) { memcpy(v, t->t.v, sizeof(t->t.v)); }      \
  PX##gctimer PX##convert_vec2gctimer(const double* v) {                                                   \
    PX##gctimer t = new PX##gctimer_s;                                                                     \
    memcpy(t->t.v, v, sizeof(t->t.v));                                                                     \
    return t;                                                                                              \
  }                                                                                                        \
  void PX##destroy_gctimer(PX##gctimer t) { delete t; }                                                    \
  }

PG_GC_API(pfft_, 1, double, pfft_complex)
PG_GC_API(pfftf_, 0, float, pfftf_complex)
