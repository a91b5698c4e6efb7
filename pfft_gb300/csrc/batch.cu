// Batched execution of many plans (of uneven sizes) in one persistent launch:
// host side (work queue, dependency counters, CUDA graph).  The kernel is in
// batch_kernel.cuh.
//
// Plans whose passes all run on the radix-8 tile go to a second queue with
// its own persistent kernel (no callee tiles: 64 registers, four CTAs per SM,
// as the stand-alone radix-8 kernel); the others (mixed-radix and general
// tiles, 80-register callees, three CTAs per SM) to the first.  The launch
// (counter reset + both kernels, the first on a forked stream) is captured
// once into a CUDA graph and replayed.
#include <stdio.h>
#include <string.h>
#include <algorithm>
#include <vector>
#include "../../include/pfft.h"
#include "../../include/pfft_gb300.h"
#include "batch_kernel.cuh"
#include "core.h"

using namespace pg;

namespace {

struct Batch {
  int arith = ARITH_DF;  // ARITH_F32 for a float batch; a double batch mixes F64 and DF plans
  std::vector<Plan*> plans;
  BatchPass* d_passes = nullptr;
  BatchTask* d_tasks = nullptr;
  unsigned* d_counters = nullptr;  // ncounters + 1 (the last is the ticket)
  int* d_err = nullptr;
  int* h_err = nullptr;  // pinned
  int ntasks = 0, ncounters = 0, threads = BATCH_THREADS, smem = 0, grid = 1;
  // the radix-8-only queue (plans whose passes all run on the radix-8 tile):
  // its own persistent kernel at four CTAs per SM, tasks after the others in
  // d_tasks, ticket word after the general queue's
  int ntasks_r8 = 0, smem_r8 = 0, grid_r8 = 0;
  int r8_kind = 1;  // k_batch's R8 for that queue: 1 any arithmetic, 2 TwoSum only, 3 block-quantised only,
                    // 4 64-bit fixed point only
  cudaStream_t side = nullptr;  // the general queue's kernel runs here when both queues are used
  cudaEvent_t fork = nullptr, join = nullptr;
  int fast_passes = 0;
  cudaStream_t stream = 0;
  bool use_graph = true;
  cudaGraphExec_t graph = nullptr;
  double bytes = 0;
};


// Counter reset, then the two persistent kernels (general queue, radix-8
// queue); when both queues have tasks the general one runs on a forked
// stream so that the two launches can overlap.
int launch_batch(Batch* b, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(b->d_counters, 0, sizeof(unsigned) * (b->ncounters + 2), s);
  if (e != cudaSuccess) return (int)e;
  e = cudaMemsetAsync(b->d_err, 0, sizeof(int), s);
  if (e != cudaSuccess) return (int)e;
  BatchLaunch q;
  q.passes = b->d_passes;
  q.counters = b->d_counters;
  q.err = b->d_err;
  q.spin_limit = 20000000LL;  // ~2 s of 100 ns naps
  const bool both = b->ntasks > 0 && b->ntasks_r8 > 0;
  int rc = 0;
  if (both) {
    if ((e = cudaEventRecord(b->fork, s)) != cudaSuccess) return (int)e;
    if ((e = cudaStreamWaitEvent(b->side, b->fork, 0)) != cudaSuccess) return (int)e;
  }
  if (b->ntasks > 0) {
    q.tasks = b->d_tasks;
    q.ntasks = b->ntasks;
    q.next = b->d_counters + b->ncounters;
    cudaStream_t sg = both ? b->side : s;
    rc = b->arith == ARITH_F32 ? batch_launch_f32(q, b->grid, b->smem, sg, 0)
                               : batch_launch_f64(q, b->grid, b->smem, sg, 0);
    if (rc) return rc;
  }
  if (b->ntasks_r8 > 0) {
    q.tasks = b->d_tasks + b->ntasks;
    q.ntasks = b->ntasks_r8;
    q.next = b->d_counters + b->ncounters + 1;
    rc = b->arith == ARITH_F32 ? batch_launch_f32(q, b->grid_r8, b->smem_r8, s, 1)
                               : batch_launch_f64(q, b->grid_r8, b->smem_r8, s, b->r8_kind);
    if (rc) return rc;
  }
  if (both) {
    if ((e = cudaEventRecord(b->join, b->side)) != cudaSuccess) return (int)e;
    if ((e = cudaStreamWaitEvent(s, b->join, 0)) != cudaSuccess) return (int)e;
  }
  return 0;
}

void free_batch(Batch* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  cudaFree(b->d_passes);
  cudaFree(b->d_tasks);
  cudaFree(b->d_counters);
  cudaFree(b->d_err);
  if (b->h_err) cudaFreeHost(b->h_err);
  delete b;
}

Batch* make_batch(Plan* const* plans, int n) {
  if (n < 1) return nullptr;
  Batch* b = new Batch();
  b->arith = plans[0] && plans[0]->arith == ARITH_F32 ? ARITH_F32 : ARITH_DF;
  std::vector<BatchPass> hp;
  std::vector<long long> ntiles;
  std::vector<int> first(n), npass(n), r8(n);
  int maxp = 0;
  const size_t fsz = b->arith == ARITH_F32 ? sizeof(float2) : sizeof(float4);
  for (int i = 0; i < n; i++) {
    Plan* pl = plans[i];
    if (!pl || (pl->arith == ARITH_F32) != (b->arith == ARITH_F32)) {
      report("batch: plans must be non-NULL and share their precision");
      free_batch(b);
      return nullptr;
    }
    b->plans.push_back(pl);
    void* bufs[4] = {pl->in, pl->out, pl->ws[0], pl->ws[1]};
    first[i] = (int)hp.size();
    npass[i] = (int)pl->fwd.passes.size();
    maxp = std::max(maxp, npass[i]);
    bool pr8 = true;  // every pass on the radix-8 tile
    int psmem = 0;
    // radix-8 / mixed-radix tile when the pass qualifies (plain c2c lines
    // of up to 512 (2^a) or 768 (3 * 2^a, 5 * 2^a) points with the same
    // orientation on both sides), else a general tile
    auto fast_tile_ok = [&](const PassParams& p, fast::FastArgs* fa, bool* ri, bool* ro) {
      const bool pow2 = !(p.N & (p.N - 1));
      return kernel_path() == 1 && p.kpath == 0 && p.N <= (pow2 ? 512 : 768) &&
             fast::fast_args(p, pl->arith, fa, ri, ro) && *ri == *ro && fa->plain;
    };
    // FX mantissas kept between passes need the radix-8 tile on both sides;
    // a plan with a linked pass that runs a general tile here gets double
    // intermediates in the batch (results within rounding of its own
    // executes instead of bit for bit)
    bool unlink = false;
    for (const Pass& ps : pl->fwd.passes) {
      fast::FastArgs fa;
      bool ri, ro;
      if ((ps.p.fx_in || ps.p.fx_out) && !fast_tile_ok(ps.p, &fa, &ri, &ro)) unlink = true;
    }
    for (const Pass& ps : pl->fwd.passes) {
      BatchPass bp;
      memset(&bp, 0, sizeof(bp));
      bp.p = ps.p;
      bp.p.src = bufs[ps.src];
      bp.p.dst = bufs[ps.dst];
      if (unlink) bp.p.fx_in = bp.p.fx_out = 0;
      cudaError_t e;
      bp.arith = pl->arith;
      bp.p.tw = twiddle_table(ps.p.M, pl->arith, &e);
      if (!bp.p.tw) {
        cuda_check(e, "batch twiddles");
        free_batch(b);
        return nullptr;
      }
      bp.done = (int)hp.size();
      bool ri = false, ro = false;
      long long tiles;
      const bool pow2 = !(ps.p.N & (ps.p.N - 1));
      // (a pass the autotuner or wisdom put on the general kernel keeps it)
      // (r2c / c2r / windowed / DCT passes keep the general tile in a batch)
      if (fast_tile_ok(bp.p, &bp.fa, &ri, &ro)) {
        bp.fastN = ps.p.N;
        bp.frow = ri ? 1 : 0;
        bp.mixed = pow2 ? 0 : 1;
        // lines per tile: BATCH_THREADS threads of N/8 (radix-8) or N/E (mixed) per line
        const int L = pow2 ? batch_fast_lines(bp.fastN)
                           : (pl->arith == ARITH_F32 ? fast::mixed_L<fast::F32>(bp.fastN) : fast::mixed_L<fast::FDD>(bp.fastN));
        tiles = (ps.p.nlines + L - 1) / L;
        const int lsp = fsz == 8 ? bp.fastN + 16 : bp.fastN + bp.fastN / 8 + 4;  // as fast_smem_bytes
        psmem = std::max(psmem, (int)((fsz == 8 ? 16 * L : (24 * L + 15) / 16 * 16) + (size_t)L * lsp * fsz));  // header: fast_hdr
        if (bp.mixed) pr8 = false;
        b->fast_passes++;
      } else {
        bp.fastN = 0;
        // the batch gets its parallelism from its many plans: start from the
        // largest tile (64 lines) and halve until it fits the block (256
        // threads) and a third of an SM's shared memory
        bp.p.L = (int)std::min<long long>(64, std::max(1LL, bp.p.nlines));
        if (!fit_pass_threads(&bp.p, pl->arith, BATCH_THREADS, 72 * 1024)) {
          report("batch: a pass needs more threads than the batched launch has");
          free_batch(b);
          return nullptr;
        }
        tiles = (bp.p.nlines + bp.p.L - 1) / bp.p.L;
        bp.small = pass_is_small(bp.p) ? 1 : 0;
        psmem = std::max(psmem, bp.p.smem_bytes);
        pr8 = false;
      }
      b->bytes += ps.bytes;
      hp.push_back(bp);
      ntiles.push_back(tiles);
    }
    r8[i] = pr8 ? 1 : 0;
    if (pr8)
      b->smem_r8 = std::max(b->smem_r8, psmem);
    else
      b->smem = std::max(b->smem, psmem);
  }
  b->ncounters = (int)hp.size();
  // two queues, each ordered by pass level (a task's dependency is the
  // previous pass of its plan, in the same queue)
  std::vector<BatchTask> tasks, tasks_r8;
  for (int lvl = 0; lvl < maxp; lvl++)
    for (int i = 0; i < n; i++) {
      if (lvl >= npass[i]) continue;
      int pi = first[i] + lvl;
      int dep = lvl > 0 ? pi - 1 : -1;
      int need = dep >= 0 ? (int)ntiles[dep] : 0;
      std::vector<BatchTask>& q = r8[i] ? tasks_r8 : tasks;
      for (long long t = 0; t < ntiles[pi]; t++) q.push_back({pi, (int)t, dep, need});
    }
  b->ntasks = (int)tasks.size();
  b->ntasks_r8 = (int)tasks_r8.size();
  // double: the radix-8 queue's kernel carries only the arithmetic its plans use
  if (b->arith != ARITH_F32) {
    bool any_q = false, any_d = false, any_x = false;
    for (int i = 0; i < n; i++)
      if (r8[i]) (plans[i]->quant == 2 ? any_x : plans[i]->quant ? any_q : any_d) = true;
    const int kinds = (int)any_q + (int)any_d + (int)any_x;
    b->r8_kind = kinds > 1 ? 1 : (any_x ? 4 : (any_q ? 3 : 2));
  }
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  for (int k = 0; k < 2; k++) {
    const int nt = k ? b->ntasks_r8 : b->ntasks;
    if (nt == 0) continue;
    const int sm = k ? b->smem_r8 : b->smem;
    const void* kfn = b->arith == ARITH_F32 ? batch_kernel_f32(k) : batch_kernel_f64(k ? b->r8_kind : 0);
    int per = 0;
    if (cuda_check(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, sm), "batch attribute") ||
        cuda_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kfn, BATCH_THREADS, sm), "batch occupancy")) {
      free_batch(b);
      return nullptr;
    }
    (k ? b->grid_r8 : b->grid) = std::max(1, std::min(nt, std::max(1, per) * nsm));
  }
  if (b->ntasks > 0 && b->ntasks_r8 > 0 &&
      (cuda_check(cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking), "batch stream") ||
       cuda_check(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "batch event") ||
       cuda_check(cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming), "batch event"))) {
    free_batch(b);
    return nullptr;
  }
  tasks.insert(tasks.end(), tasks_r8.begin(), tasks_r8.end());
  if (cuda_check(cudaMalloc(&b->d_passes, sizeof(BatchPass) * hp.size()), "batch alloc") ||
      cuda_check(cudaMalloc(&b->d_tasks, sizeof(BatchTask) * std::max<size_t>(1, tasks.size())), "batch alloc") ||
      cuda_check(cudaMalloc(&b->d_counters, sizeof(unsigned) * (b->ncounters + 2)), "batch alloc") ||
      cuda_check(cudaMalloc(&b->d_err, sizeof(int)), "batch alloc") ||
      cuda_check(cudaMallocHost(&b->h_err, sizeof(int)), "batch alloc")) {
    free_batch(b);
    return nullptr;
  }
  cudaMemcpy(b->d_passes, hp.data(), sizeof(BatchPass) * hp.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(b->d_tasks, tasks.data(), sizeof(BatchTask) * tasks.size(), cudaMemcpyHostToDevice);
  return b;
}

int run_batch(Batch* b) {
  cudaStream_t s = b->stream;
  int rc;
  if (b->use_graph) {
    if (!b->graph) {
      cudaStream_t cs;
      if (cuda_check(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "batch graph stream")) return -1;
      cudaGraph_t g;
      cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
      rc = launch_batch(b, cs);
      cudaError_t ce = cudaStreamEndCapture(cs, &g);
      cudaStreamDestroy(cs);
      if (rc || ce != cudaSuccess) return cuda_check(rc ? (cudaError_t)rc : ce, "batch graph capture");
      ce = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      if (cuda_check(ce, "batch graph instantiate")) return -1;
    }
    rc = (int)cudaGraphLaunch(b->graph, s);
  } else {
    rc = launch_batch(b, s);
  }
  if (rc) return cuda_check((cudaError_t)rc, "batch launch");
  rc = (int)cudaMemcpyAsync(b->h_err, b->d_err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (rc) return cuda_check((cudaError_t)rc, "batch status");
  rc = (int)cudaStreamSynchronize(s);
  if (rc) return cuda_check((cudaError_t)rc, "batch execute");
  if (*b->h_err) {
    report("batch: a dependency wait timed out");
    return -2;
  }
  return 0;
}

}  // namespace

struct pfft_gb300_batch_s {
  Batch* b;
};

struct pfft_plan_s {
  Plan* p;
};
struct pfftf_plan_s {
  Plan* p;
};

extern "C" {

pfft_gb300_batch pfft_gb300_batch_create(int nplans, const pfft_plan* plans) {
  std::vector<Plan*> v;
  for (int i = 0; i < nplans; i++) v.push_back(plans[i] ? plans[i]->p : nullptr);
  Batch* b = make_batch(v.data(), nplans);
  if (!b) return nullptr;
  return new pfft_gb300_batch_s{b};
}

pfft_gb300_batch pfftf_gb300_batch_create(int nplans, const pfftf_plan* plans) {
  std::vector<Plan*> v;
  for (int i = 0; i < nplans; i++) v.push_back(plans[i] ? plans[i]->p : nullptr);
  Batch* b = make_batch(v.data(), nplans);
  if (!b) return nullptr;
  return new pfft_gb300_batch_s{b};
}

int pfft_gb300_batch_execute(pfft_gb300_batch batch) {
  if (!batch) return -1;
  return run_batch(batch->b);
}

int pfft_gb300_batch_set_stream(pfft_gb300_batch batch, void* stream) {
  if (!batch) return -1;
  batch->b->stream = (cudaStream_t)stream;
  return 0;
}

int pfft_gb300_batch_set_graph(pfft_gb300_batch batch, int on) {
  if (!batch) return -1;
  batch->b->use_graph = on != 0;
  return 0;
}

int pfft_gb300_batch_info(pfft_gb300_batch batch, int* ntasks, int* grid, int* threads, double* bytes) {
  if (!batch) return -1;
  if (ntasks) *ntasks = batch->b->ntasks + batch->b->ntasks_r8;
  if (grid) *grid = (batch->b->ntasks ? batch->b->grid : 0) + (batch->b->ntasks_r8 ? batch->b->grid_r8 : 0);
  if (threads) *threads = batch->b->threads;
  if (bytes) *bytes = batch->b->bytes;
  return 0;
}

void pfft_gb300_batch_destroy(pfft_gb300_batch batch) {
  if (!batch) return;
  free_batch(batch->b);
  delete batch;
}

// Runs the batch kernel on a one-task queue whose dependency counter nothing
// increments, with a wait limit of `spin_limit` naps: the wait must expire,
// the kernel must return, and the status must be -2 (timed out).  Used by the
// tests to exercise the bounded wait without hanging anything.
int pfft_gb300_batch_wait_selftest(long long spin_limit) {
  BatchPass* dp = nullptr;
  BatchTask* dt = nullptr;
  unsigned* dc = nullptr;
  int* de = nullptr;
  int herr = 0, rc = 0;
  BatchPass hp;
  memset(&hp, 0, sizeof(hp));
  hp.p.nlines = 0;  // an empty tile: nothing is read or written
  hp.p.L = 1;
  hp.p.M = 1;
  hp.p.N = 1;
  hp.p.sign = -1;
  hp.done = 0;
  BatchTask ht = {0, 0, 1, 1};  // waits for counter 1 to reach 1: never happens
  if (cudaMalloc(&dp, sizeof(hp)) != cudaSuccess || cudaMalloc(&dt, sizeof(ht)) != cudaSuccess ||
      cudaMalloc(&dc, 3 * sizeof(unsigned)) != cudaSuccess || cudaMalloc(&de, sizeof(int)) != cudaSuccess) {
    rc = -1;
  } else {
    cudaMemcpy(dp, &hp, sizeof(hp), cudaMemcpyHostToDevice);
    cudaMemcpy(dt, &ht, sizeof(ht), cudaMemcpyHostToDevice);
    cudaMemset(dc, 0, 3 * sizeof(unsigned));
    cudaMemset(de, 0, sizeof(int));
    BatchLaunch q;
    q.passes = dp;
    q.tasks = dt;
    q.ntasks = 1;
    q.counters = dc;
    q.next = dc + 2;
    q.err = de;
    q.spin_limit = spin_limit;
    if (batch_launch_f32(q, 1, 1024, 0) != 0 || cudaDeviceSynchronize() != cudaSuccess) rc = -1;
    cudaMemcpy(&herr, de, sizeof(int), cudaMemcpyDeviceToHost);
    if (!rc) rc = herr ? -2 : 0;
  }
  cudaFree(dp);
  cudaFree(dt);
  cudaFree(dc);
  cudaFree(de);
  return rc;
}

}  // extern "C"
