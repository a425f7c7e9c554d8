// The runtime around the fill: the launch-option autotuner and the CUDA
// graph of RK4 steps of a batch of forests.
//
// The reference has neither: its device fill is one KernelAbstractions launch
// per group with the default workgroup (src/ghosts.jl:420-521), and its time
// integration replays every launch from the host each step.  Here the tuner
// times every candidate of a schedule's launch options on the caller's own
// data, and the RK4 step of the wave equation (four fills and four fused
// stages) is captured once and replayed as one graph launch.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <new>
#include <string>

#include "tam_internal.h"
#include "treeamr_cuda.h"

struct tam_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int device = 0;
};

namespace {

struct Guard {
  int prev = -1;
  bool ok = false;
  explicit Guard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) return;
    ok = prev == dev || cudaSetDevice(dev) == cudaSuccess;
  }
  ~Guard() {
    if (ok && prev >= 0) cudaSetDevice(prev);
  }
};

// Best of `reps` fills on `stream` after one warm-up, in milliseconds, or a
// negative status.
double time_fill(tam_sched *s, void *work, int32_t nvars, int64_t nblocks,
                 const void *factors, int32_t reps, cudaStream_t stream, cudaEvent_t a,
                 cudaEvent_t b, int *rc) {
  *rc = tam_fill(s, work, nvars, nblocks, factors, TAM_STAGE_ALL_FIRST, TAM_STAGE_ALL_LAST,
                 stream);
  if (*rc != TAM_OK) return -1.0;
  double best = 1e300;
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(a, stream);
    *rc = tam_fill(s, work, nvars, nblocks, factors, TAM_STAGE_ALL_FIRST, TAM_STAGE_ALL_LAST,
                   stream);
    if (*rc != TAM_OK) return -1.0;
    cudaEventRecord(b, stream);
    if (cudaEventSynchronize(b) != cudaSuccess) {
      *rc = TAM_ECUDA;
      return -1.0;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    best = std::min(best, (double)ms);
  }
  return best;
}

}  // namespace

extern "C" {

int tam_autotune(tam_sched *s, void *work, int32_t nvars, int64_t nblocks, const void *factors,
                 int32_t reps, void *stream, int64_t *tile_items, int64_t *threads,
                 int64_t *int_mul, double *best_ms) {
  if (!s || !work) return TAM_EINVAL;
  if (reps < 1) reps = 1;
  int64_t old_t, old_th, old_im;
  tam_schedule_get_option(s, TAM_OPT_TILE_ITEMS, &old_t);
  tam_schedule_get_option(s, TAM_OPT_THREADS, &old_th);
  tam_schedule_get_option(s, TAM_OPT_INT_MUL, &old_im);
  static const int kTiles[] = {32, 64, 128, 256, 512};
  static const int kThreads[] = {128, 256, 512};
  // the integer-pipe multiply is a Float64 path; Float32 has one candidate
  const int dtype_f64 = s->dtype == TAM_F64 ? 1 : 0;
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    if (a) cudaEventDestroy(a);
    return TAM_ECUDA;
  }
  double best = 1e300;
  int bt = (int)old_t, bth = (int)old_th, bim = (int)old_im;
  int rc = TAM_OK;
  // every combination: the best tile and CTA size differ between the two
  // multiply paths, so neither is chosen before the other
  for (int im = 0; im <= (int)dtype_f64 && rc == TAM_OK; ++im)
    for (int t : kTiles)
      for (int th : kThreads) {
        if ((rc = tam_schedule_set_option(s, TAM_OPT_INT_MUL, im)) != TAM_OK ||
            (rc = tam_schedule_set_option(s, TAM_OPT_TILE_ITEMS, t)) != TAM_OK ||
            (rc = tam_schedule_set_option(s, TAM_OPT_THREADS, th)) != TAM_OK)
          break;
        const double ms =
            time_fill(s, work, nvars, nblocks, factors, reps, (cudaStream_t)stream, a, b, &rc);
        if (rc != TAM_OK) break;
        if (ms < best) {
          best = ms;
          bt = t;
          bth = th;
          bim = im;
        }
      }
  // then the work's grouping and order, one option at a time from the best
  // so far: stage groups as one launch or stage by stage, stencil tiles by
  // path or by block, large stencil boxes staged in shared memory or read in
  // place, Float64 variables a lane, the blocks' visiting order, points a
  // lane of the copy kernel, the copies' share of the machine beside the
  // stencils
  int64_t old_pt = 0, old_bo = 0, old_cp = 1, old_ms = 1, old_sg = 0, old_pv = 0, old_cs = 0;
  int64_t old_sa = 0, old_st = 0;
  tam_schedule_get_option(s, TAM_OPT_PATH_TILES, &old_pt);
  tam_schedule_get_option(s, TAM_OPT_BLOCK_ORDER, &old_bo);
  tam_schedule_get_option(s, TAM_OPT_COPY_POINTS, &old_cp);
  tam_schedule_get_option(s, TAM_OPT_MERGE_STAGES, &old_ms);
  tam_schedule_get_option(s, TAM_OPT_STAGED, &old_sg);
  tam_schedule_get_option(s, TAM_OPT_PAIR_VARS, &old_pv);
  tam_schedule_get_option(s, TAM_OPT_COPY_SHARE, &old_cs);
  tam_schedule_get_option(s, TAM_OPT_SOFT_ADD, &old_sa);
  tam_schedule_get_option(s, TAM_OPT_STENCIL_TILE, &old_st);
  if (rc == TAM_OK) {
    (void)((rc = tam_schedule_set_option(s, TAM_OPT_INT_MUL, bim)) == TAM_OK &&
           (rc = tam_schedule_set_option(s, TAM_OPT_TILE_ITEMS, bt)) == TAM_OK &&
           (rc = tam_schedule_set_option(s, TAM_OPT_THREADS, bth)) == TAM_OK);
  }
  struct Dim {
    int32_t option;
    int values[4];
    int n;
    int64_t best;
  } dims[] = {{TAM_OPT_MERGE_STAGES, {1, 0, 0}, 2, old_ms},
              {TAM_OPT_PATH_TILES, {0, 1, 0}, 2, old_pt},
              {TAM_OPT_STAGED, {0, 1, 0}, 2, old_sg},
              {TAM_OPT_PAIR_VARS, {0, 1, 0}, dtype_f64 ? 2 : 1, old_pv},
              {TAM_OPT_BLOCK_ORDER, {0, 1, 2, 3}, 4, old_bo},
              {TAM_OPT_COPY_POINTS, {1, 2, 4}, 3, old_cp},
              {TAM_OPT_COPY_SHARE, {0, 1, 2, 4}, 4, old_cs},
              {TAM_OPT_SOFT_ADD, {0, 1, 0, 0}, dtype_f64 ? 2 : 1, old_sa},
              {TAM_OPT_STENCIL_TILE, {0, 32, 64, 128}, 4, old_st}};
  // two sweeps: the options interact (the copies' share of the machine and
  // the stencils' tiling, for one), so the second revisits each from the
  // others' best
  for (int sweep = 0; sweep < 2; ++sweep) {
    for (Dim &dm : dims) {
      for (int i = 0; i < dm.n && rc == TAM_OK; ++i) {
        if (sweep == 1 && dm.values[i] == dm.best) continue;
        if ((rc = tam_schedule_set_option(s, dm.option, dm.values[i])) != TAM_OK) break;
        const double ms =
            time_fill(s, work, nvars, nblocks, factors, reps, (cudaStream_t)stream, a, b, &rc);
        if (rc != TAM_OK) break;
        if (ms < best) {
          best = ms;
          dm.best = dm.values[i];
        }
      }
      if (rc == TAM_OK) rc = tam_schedule_set_option(s, dm.option, dm.best);
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  // leave the best (or, after a failure, the options the call found)
  if (rc != TAM_OK) {
    tam_schedule_set_option(s, TAM_OPT_INT_MUL, old_im);
    tam_schedule_set_option(s, TAM_OPT_TILE_ITEMS, old_t);
    tam_schedule_set_option(s, TAM_OPT_THREADS, old_th);
    tam_schedule_set_option(s, TAM_OPT_PATH_TILES, old_pt);
    tam_schedule_set_option(s, TAM_OPT_BLOCK_ORDER, old_bo);
    tam_schedule_set_option(s, TAM_OPT_COPY_POINTS, old_cp);
    tam_schedule_set_option(s, TAM_OPT_MERGE_STAGES, old_ms);
    tam_schedule_set_option(s, TAM_OPT_STAGED, old_sg);
    tam_schedule_set_option(s, TAM_OPT_PAIR_VARS, old_pv);
    tam_schedule_set_option(s, TAM_OPT_COPY_SHARE, old_cs);
    tam_schedule_set_option(s, TAM_OPT_SOFT_ADD, old_sa);
    tam_schedule_set_option(s, TAM_OPT_STENCIL_TILE, old_st);
    return rc;
  }
  if (tile_items) *tile_items = bt;
  if (threads) *threads = bth;
  if (int_mul) *int_mul = bim;
  if (best_ms) *best_ms = best;
  return TAM_OK;
}

int tam_graph_capture_rk4(tam_batch *b, int32_t dtype, const tam_wave_block *blocks,
                          int32_t nblocks, int32_t max_points_per_block, void *y, void *ta,
                          void *tb, void *acc, int64_t arena_elems, int32_t nvars,
                          const void *factor_arena, int64_t factor_elems, double dt,
                          int32_t steps, int32_t device, tam_graph **out) {
  if (!b || !blocks || !y || !ta || !tb || !acc || !out || steps < 1) return TAM_EINVAL;
  *out = nullptr;
  Guard guard(device);
  if (!guard.ok) return TAM_ECUDA;
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return TAM_ECUDA;
  // the RK4 step (Butcher tableau 0, 1/2, 1/2, 1; weights 1/6, 1/3, 1/3, 1/6):
  // each fill followed by one fused stage that forms the next stage state
  // and adds the stage's share of the step
  auto step = [&]() -> int {
    int rc;
    if ((rc = tam_batch_fill(b, y, arena_elems, nvars, factor_arena, factor_elems,
                             TAM_STAGE_ALL_FIRST, TAM_STAGE_ALL_LAST, st)) != TAM_OK ||
        (rc = tam_wave_rk4_stage(dtype, blocks, nblocks, max_points_per_block, y, y, ta,
                                 nullptr, acc, dt / 2, dt / 6, st)) != TAM_OK ||
        (rc = tam_batch_fill(b, ta, arena_elems, nvars, factor_arena, factor_elems,
                             TAM_STAGE_ALL_FIRST, TAM_STAGE_ALL_LAST, st)) != TAM_OK ||
        (rc = tam_wave_rk4_stage(dtype, blocks, nblocks, max_points_per_block, ta, y, tb, acc,
                                 acc, dt / 2, dt / 3, st)) != TAM_OK ||
        (rc = tam_batch_fill(b, tb, arena_elems, nvars, factor_arena, factor_elems,
                             TAM_STAGE_ALL_FIRST, TAM_STAGE_ALL_LAST, st)) != TAM_OK ||
        (rc = tam_wave_rk4_stage(dtype, blocks, nblocks, max_points_per_block, tb, y, ta, acc,
                                 acc, dt, dt / 3, st)) != TAM_OK ||
        (rc = tam_batch_fill(b, ta, arena_elems, nvars, factor_arena, factor_elems,
                             TAM_STAGE_ALL_FIRST, TAM_STAGE_ALL_LAST, st)) != TAM_OK ||
        (rc = tam_wave_rk4_stage(dtype, blocks, nblocks, max_points_per_block, ta, y, nullptr,
                                 acc, y, 0.0, dt / 6, st)) != TAM_OK)
      return rc;
    return TAM_OK;
  };
  tam_graph *g = new (std::nothrow) tam_graph;
  if (!g) {
    cudaStreamDestroy(st);
    return TAM_ENOMEM;
  }
  g->device = device;
  int rc = TAM_OK;
  // every launch is captured, none runs: the arrays are not touched here
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    for (int32_t i = 0; i < steps && rc == TAM_OK; ++i) rc = step();
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(st, &graph);
    g->graph = graph;
    if (rc == TAM_OK && e == cudaSuccess)
      e = cudaGraphInstantiate(&g->exec, graph, 0);
  }
  cudaStreamDestroy(st);
  if (rc != TAM_OK || e != cudaSuccess) {
    cudaGetLastError();
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return rc != TAM_OK ? rc : TAM_ECUDA;
  }
  *out = g;
  return TAM_OK;
}

int tam_graph_launch(tam_graph *g, void *stream) {
  if (!g || !g->exec) return TAM_EINVAL;
  Guard guard(g->device);
  if (!guard.ok) return TAM_ECUDA;
  return cudaGraphLaunch(g->exec, (cudaStream_t)stream) == cudaSuccess ? TAM_OK : TAM_ECUDA;
}

void tam_graph_free(tam_graph *g) {
  if (!g) return;
  Guard guard(g->device);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
}

}  // extern "C"
