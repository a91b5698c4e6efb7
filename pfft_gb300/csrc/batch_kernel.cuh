// Persistent kernel of the batched execution (host side: batch.cu).
//
// Every pass of every plan is cut into tiles; the tiles form one work queue,
// ordered by pass level (all first passes, then all second passes, ...).  A
// fixed grid of CTAs pulls tiles with an atomic ticket; a tile of pass i of
// plan p first waits until all tiles of pass i-1 of the same plan are done (a
// per-(plan, pass) counter), runs the tile, then publishes its stores (fence)
// and bumps its own counter.  Tiles are dequeued in order, so every tile a
// waiting CTA depends on is already held by a running CTA: the queue cannot
// deadlock.  Each wait is bounded; on expiry the kernel records an error word
// (read by the host) and carries on instead of spinning forever.  Reads of
// data produced inside the launch go through L2 only (ld.global.cg), so no SM
// can see a stale L1 line.
//
// A tile is either a register-resident radix-8 tile (power-of-two c2c lines
// of 16..512 points, BATCH_THREADS = L * N/8 threads) or a general pass tile.
// The batch_*.cu units are compiled as relocatable device code.
#pragma once
#include <type_traits>
#include "fft_fast.cuh"
#include "fft_mixed.cuh"
#include "pass_tile.cuh"

namespace pg {

constexpr int BATCH_THREADS = 256;

struct BatchTask {
  int pass;   // index into the pass array
  int tile;   // tile of that pass
  int dep;    // counter to wait for (-1: none)
  int need;   // value it must reach
};

struct BatchPass {
  PassParams p;      // general tile parameters
  fast::FastArgs fa; // radix-8 tile parameters (fastN > 0)
  int fastN;         // line length of a radix-8 tile pass, 0 for a general tile
  int frow;          // radix-8 tile: 1 = lines contiguous on both sides, 0 = columns
  int done;          // counter this pass increments
  int arith;         // arithmetic of the pass's plan
  int small;         // general tile of a c2c pass with radices <= 8 (pass_is_small)
  int mixed;         // fastN is a 3 * 2^a or 5 * 2^a length: mixed-radix tile
};

struct BatchLaunch {
  const BatchPass* passes;
  const BatchTask* tasks;
  int ntasks;
  unsigned* counters;
  unsigned* next;
  int* err;
  long long spin_limit;
};

// lines per radix-8 tile at BATCH_THREADS threads
__host__ __device__ constexpr int batch_fast_lines(int N) { return BATCH_THREADS * 8 / N; }

// Radix-8 tiles are expanded inline (they are register-resident and short);
// the general tiles are separate device functions in their own translation
// units (batch_tiles_gen_*.cu, relocatable device code, at most 80 registers
// so that three 256-thread blocks fit an SM): each is compiled once, in
// parallel with the rest of the build.
#define PG_BT_GEN(name) __device__ void name(const PassParams& p, long long tile, unsigned char* sm)
PG_BT_GEN(bt_gen_f32_m);
PG_BT_GEN(bt_gen_f32_p);
PG_BT_GEN(bt_gen_df_m);
PG_BT_GEN(bt_gen_df_p);
PG_BT_GEN(bt_gen_f64_m);
PG_BT_GEN(bt_gen_f64_p);
PG_BT_GEN(bt_small_f32_m);
PG_BT_GEN(bt_small_f32_p);
PG_BT_GEN(bt_small_df_m);
PG_BT_GEN(bt_small_df_p);
PG_BT_GEN(bt_small_f64_m);
PG_BT_GEN(bt_small_f64_p);
#define PG_BT_DEF_GEN(name, A, SIGN) \
  PG_BT_GEN(name) { pass_tile<A, SIGN, true>(p, tile, sm); }
#define PG_BT_DEF_SMALL(name, A, SIGN) \
  PG_BT_GEN(name) { pass_tile<A, SIGN, true, true>(p, tile, sm); }

template <class P, int N>
__device__ __forceinline__ void batch_fast_n(const BatchPass& bp, long long tile, unsigned char* sm) {
  constexpr int L = batch_fast_lines(N);
  if (bp.frow) {
    if (bp.p.sign < 0)
      fast::fast_tile<P, -1, N, L, true, true, true>(bp.fa, tile, sm);
    else
      fast::fast_tile<P, 1, N, L, true, true, true>(bp.fa, tile, sm);
  } else {
    if (bp.p.sign < 0)
      fast::fast_tile<P, -1, N, L, false, false, true>(bp.fa, tile, sm);
    else
      fast::fast_tile<P, 1, N, L, false, false, true>(bp.fa, tile, sm);
  }
}

template <class P>
__device__ __forceinline__ void batch_fast_p(const BatchPass& bp, long long tile, unsigned char* sm) {
  switch (bp.fastN) {
    case 16: batch_fast_n<P, 16>(bp, tile, sm); break;
    case 32: batch_fast_n<P, 32>(bp, tile, sm); break;
    case 64: batch_fast_n<P, 64>(bp, tile, sm); break;
    case 128: batch_fast_n<P, 128>(bp, tile, sm); break;
    case 256: batch_fast_n<P, 256>(bp, tile, sm); break;
    default: batch_fast_n<P, 512>(bp, tile, sm); break;
  }
}

// double batches: the arithmetic of the pass's plan (PassParams::quant: 64-bit
// fixed point for double plans, TwoSum or block-quantised float-float
// radix-8 stages for float-float plans)
template <bool DOUBLE>
__device__ __forceinline__ void batch_fast(const BatchPass& bp, long long tile, unsigned char* sm) {
  if constexpr (DOUBLE) {
    if (bp.p.quant == 2)
      batch_fast_p<fast::FX>(bp, tile, sm);
    else if (bp.p.quant)
      batch_fast_p<fast::FQ>(bp, tile, sm);
    else
      batch_fast_p<fast::FDD>(bp, tile, sm);
  } else {
    batch_fast_p<fast::F32>(bp, tile, sm);
  }
}

// Mixed-radix tiles (3 * 2^a and 5 * 2^a lengths), callee units
// batch_tiles_mixed_<arith>_<family>.cu, 80 registers like the general tiles.
#define PG_BT_MX(name) __device__ void name(const fast::FastArgs& a, long long tile, unsigned char* sm)
// the four tiles of a length: rows / columns, forward / backward
#define PG_BT_MX4(P, N) \
  PG_BT_MX(bt_mx_##P##_##N##_rm); \
  PG_BT_MX(bt_mx_##P##_##N##_rp); \
  PG_BT_MX(bt_mx_##P##_##N##_cm); \
  PG_BT_MX(bt_mx_##P##_##N##_cp)
#define PG_BT_MX_ALL(P)                                                                                    \
  PG_BT_MX4(P, 24); PG_BT_MX4(P, 48); PG_BT_MX4(P, 96); PG_BT_MX4(P, 192); PG_BT_MX4(P, 384); PG_BT_MX4(P, 768); \
  PG_BT_MX4(P, 40); PG_BT_MX4(P, 80); PG_BT_MX4(P, 160); PG_BT_MX4(P, 320); PG_BT_MX4(P, 640)
PG_BT_MX_ALL(F32);
PG_BT_MX_ALL(FDD);
PG_BT_MX_ALL(FQ);
PG_BT_MX_ALL(FX);
#define PG_BT_DEF_MX(P, N)                                                                                       \
  PG_BT_MX(bt_mx_##P##_##N##_rm) { fast::mixed_tile<fast::P, -1, N, fast::mixed_L<fast::P>(N), true, true, true>(a, tile, sm); }   \
  PG_BT_MX(bt_mx_##P##_##N##_rp) { fast::mixed_tile<fast::P, 1, N, fast::mixed_L<fast::P>(N), true, true, true>(a, tile, sm); }    \
  PG_BT_MX(bt_mx_##P##_##N##_cm) { fast::mixed_tile<fast::P, -1, N, fast::mixed_L<fast::P>(N), false, false, true>(a, tile, sm); } \
  PG_BT_MX(bt_mx_##P##_##N##_cp) { fast::mixed_tile<fast::P, 1, N, fast::mixed_L<fast::P>(N), false, false, true>(a, tile, sm); }

// one of the four tiles of policy P and length N
#define PG_BT_MX_CALL(P, N)                                                    \
  do {                                                                         \
    if (bp.frow)                                                               \
      neg ? bt_mx_##P##_##N##_rm(bp.fa, tile, sm) : bt_mx_##P##_##N##_rp(bp.fa, tile, sm); \
    else                                                                       \
      neg ? bt_mx_##P##_##N##_cm(bp.fa, tile, sm) : bt_mx_##P##_##N##_cp(bp.fa, tile, sm); \
  } while (0)
// double batches: the arithmetic of the pass's plan (PassParams::quant)
#define PG_BT_MX_CASE(N)                 \
  case N:                                \
    if (!DOUBLE)                         \
      PG_BT_MX_CALL(F32, N);             \
    else if (bp.p.quant == 2)            \
      PG_BT_MX_CALL(FX, N);              \
    else if (bp.p.quant)                 \
      PG_BT_MX_CALL(FQ, N);              \
    else                                 \
      PG_BT_MX_CALL(FDD, N);             \
    break

template <bool DOUBLE>
__device__ __forceinline__ void batch_mixed(const BatchPass& bp, long long tile, unsigned char* sm) {
  const bool neg = bp.p.sign < 0;
  switch (bp.fastN) {
    PG_BT_MX_CASE(24);
    PG_BT_MX_CASE(48);
    PG_BT_MX_CASE(96);
    PG_BT_MX_CASE(192);
    PG_BT_MX_CASE(384);
    PG_BT_MX_CASE(768);
    PG_BT_MX_CASE(40);
    PG_BT_MX_CASE(80);
    PG_BT_MX_CASE(160);
    PG_BT_MX_CASE(320);
    PG_BT_MX_CASE(640);
  }
}

// Float batches (DOUBLE = false) run FP32 tiles; in a double batch every
// pass carries its own arithmetic (native FP64 for small plans, float-float
// for large ones).  R8 > 0: the queue holds radix-8 tiles only (plans whose
// passes all run on the radix-8 tile); that kernel carries no callee tiles
// and fits four CTAs per SM (64 registers, the stand-alone kernel's budget)
// instead of three.  R8 = 1 carries every double arithmetic, 2 only the
// TwoSum tiles, 3 only the block-quantised ones, 4 only the 64-bit
// fixed-point ones (fewer code paths for the register allocator).
template <bool DOUBLE, int R8>
__global__ void __launch_bounds__(BATCH_THREADS, R8 ? 4 : 3) k_batch(const BatchLaunch q) {
  extern __shared__ __align__(16) unsigned char smraw[];
  __shared__ int s_task;
  if (threadIdx.x == 0) s_task = (int)atomicAdd(q.next, 1u);
  __syncthreads();
  for (;;) {
    const int t = s_task;
    if (t >= q.ntasks) break;
    // the next ticket is taken now, so that its round trip overlaps this tile
    int next_t = 0;
    if (threadIdx.x == 0) next_t = (int)atomicAdd(q.next, 1u);
    const BatchTask task = q.tasks[t];
    const BatchPass& bp = q.passes[task.pass];
    if (task.dep >= 0) {
      if (threadIdx.x == 0) {
        volatile unsigned* c = q.counters + task.dep;
        long long it = 0;
        while (*c < (unsigned)task.need) {
          if (++it > q.spin_limit) {
            atomicExch(q.err, 1);
            break;
          }
          __nanosleep(100);
        }
        __threadfence();
      }
      __syncthreads();
    }
    const long long tile = task.tile;
    unsigned char* sm = smraw;
    const bool neg = bp.p.sign < 0;
    if constexpr (R8 == 4 && DOUBLE) {
      batch_fast_p<fast::FX>(bp, tile, sm);
    } else if constexpr (R8 == 3 && DOUBLE) {
      batch_fast_p<fast::FQ>(bp, tile, sm);
    } else if constexpr (R8 == 2 && DOUBLE) {
      batch_fast_p<fast::FDD>(bp, tile, sm);
    } else if constexpr (R8 > 0) {
      batch_fast<DOUBLE>(bp, tile, sm);
    } else if (bp.fastN > 0 && bp.mixed) {
      batch_mixed<DOUBLE>(bp, tile, sm);
    } else if (bp.fastN > 0) {
      batch_fast<DOUBLE>(bp, tile, sm);
    } else if (!DOUBLE) {
      if (bp.small)
        neg ? bt_small_f32_m(bp.p, tile, sm) : bt_small_f32_p(bp.p, tile, sm);
      else
        neg ? bt_gen_f32_m(bp.p, tile, sm) : bt_gen_f32_p(bp.p, tile, sm);
    } else if (bp.arith == ARITH_F64) {
      if (bp.small)
        neg ? bt_small_f64_m(bp.p, tile, sm) : bt_small_f64_p(bp.p, tile, sm);
      else
        neg ? bt_gen_f64_m(bp.p, tile, sm) : bt_gen_f64_p(bp.p, tile, sm);
    } else {
      if (bp.small)
        neg ? bt_small_df_m(bp.p, tile, sm) : bt_small_df_p(bp.p, tile, sm);
      else
        neg ? bt_gen_df_m(bp.p, tile, sm) : bt_gen_df_p(bp.p, tile, sm);
    }
    // publish: every thread's stores are ordered before thread 0's fence by
    // the barrier, the fence makes them visible at device scope before the
    // counter increment (release pattern; the waiting side loads the counter,
    // fences, then synchronises its block)
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(q.counters + bp.done, 1u);
      s_task = next_t;
    }
    __syncthreads();
  }
}

// instantiation units batch_f32.cu / batch_f64.cu (r8: the radix-8-only
// kernel variant, k_batch's R8; float batches have variants 0 and 1)
int batch_launch_f32(const BatchLaunch& q, int grid, int smem, cudaStream_t s, int r8 = 0);
int batch_launch_f64(const BatchLaunch& q, int grid, int smem, cudaStream_t s, int r8 = 0);
const void* batch_kernel_f32(int r8 = 0);
const void* batch_kernel_f64(int r8 = 0);

}  // namespace pg
