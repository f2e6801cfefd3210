// af3d_capi.cu -- host side of the C ABI declared in include/af3d.h.
//
// The context owns every device buffer; the reference's caller-owned arrays become planes of a
// structure-of-arrays state kept in cell-sorted order.  A context holds one flume (the plain
// drop-in) or many independent flumes (a batched ensemble) that share dt and the clock; every
// flume has its own system_par, Funnel and cell grid, and the cell list is segmented by flume.
// The per-routine entry points enqueue one kernel (or the cell build) each on the context stream
// and return; af3d_step() enqueues whole fused steps and replays them from CUDA graphs.
// Device-side checks raise bits in a status word that af3d_step() and af3d_get_status() read
// back; nothing calls exit().
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "af3d_internal.h"

using namespace af3d;

namespace {

thread_local std::string g_last_error;

af3d_status fail(af3d_status code, const std::string &msg) {
  g_last_error = msg;
  return code;
}

#define AF3D_CUDA(call)                                                                         \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return fail(AF3D_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));          \
  } while (0)

constexpr long kRegridEvery = 2000;   // avalanche_hst.cu:470 and :713 (cc % 2000 == 0)
constexpr long kKernelsPerCellBuild = 5;   // predict/keys, scan, scatter, rank, permute
constexpr long kKernelsPerForcePass = 1;   // lists and forces in one kernel
#ifndef AF3D_HOST_PARTS
#define AF3D_HOST_PARTS 4
#endif
constexpr int kHostParts = AF3D_HOST_PARTS;   // af3d_step_host: parts whose copies overlap the step
constexpr long kKernelsPerStep = kKernelsPerCellBuild + 1 + kKernelsPerForcePass;   // + time advance
constexpr long kKernelsPerKeptStep = kKernelsPerStep - 1;    // a step without the permutation
constexpr long kKernelsPerRegrid = 4;
// The clumps are moved into (cell, id) order by a permutation of every plane at most this many
// steps apart (the context's `resort_every`, by default kResortEvery); the steps in between keep
// the slot order and reach the sorted order through the sort's index array.  Results do not
// depend on it (every sum runs in (sph_id, cell, id) order); it bounds how far the slot order
// may drift from the spatial order.  A long captured graph covers one such period (its first
// step permutes), so the interval is even (the pointer period of the plane sets is 2).
constexpr long kResortEvery = 64;
constexpr long kResortChoices[] = {16, 32, 64, 128, 256};   // what af3d_autotune times

// Pointer state of the context that a captured sequence of steps depends on and changes.
struct PtrState {
  Planes cur, alt;
  long long *id_cur, *id_alt;
  int *fl_cur, *fl_alt;
  NbrRec *nbr, *nbr_next;
  CullRec *cull, *cull_next;
  bool look;
};

struct StepGraph {
  PtrState start{}, end{};      // before and after the captured steps
  long steps = 0;
  bool resort_first = false;    // the first captured step permutes the planes
  bool look_last = false;       // the last captured force pass looks ahead
  cudaGraphExec_t exec = nullptr;
};

}  // namespace

namespace {

// The force kernel's shape whose last wave of blocks is fullest for n clumps on `sms` SMs: a
// launch of b blocks on sms * minb resident slots runs ceil(b / slots) waves, and the work of
// b / slots of them; fewer blocks than slots: the shape that spreads them over more SMs.  Ties
// keep the larger block.  af3d_autotune measures instead.
int force_shape_for(long n, int sms) {
  if (n <= 0 || sms <= 0) return 0;
  int best = 0;
  double best_fill = -1.0;
  for (int i = 0; i < kForceShapes; i++) {
    if (!kForceShapeDefault[i]) continue;
    const double blocks = (double)((n + kForceShapeBlock[i] - 1) / kForceShapeBlock[i]);
    const double slots = (double)sms * kForceShapeMinb[i];
    const double waves = blocks / slots;
    const double fill = waves >= 1.0 ? waves / std::ceil(waves) : std::min(blocks, (double)sms) / sms;
    if (fill > best_fill + 1e-9) {
      best_fill = fill;
      best = i;
    }
  }
  return best;
}

}  // namespace

struct af3d_ctx {
  int device = 0;
  long n = 0;
  int nflumes = 1;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  std::vector<af3d_system_par> sys;   // host mirrors, one per flume (time: see `time`)
  std::vector<af3d_funnel> fun;
  std::vector<af3d_cell_par> grid;    // refreshed from the device after device re-grids
  std::vector<long> first_id;         // ids of flume f: [first_id[f], first_id[f+1])
  double time = 0.0;                  // the shared clock, mirrored
  bool have_grid = false;
  long ntags = 9;
  int phase = AF3D_PHASE_AVALANCHE;
  int variant = AF3D_FRICTION_HST;
  int fp_mode = AF3D_FP_EXACT;
  int force_shape = 0;       // index into kForceShapeBlock / kForceShapeMinb
  double obj_length = 0.0;   // objective of af3d_adjoint: 0 deposit centroid, > 0 runout length scale
  long cc = 0;                        // steps done in the current phase
  bool imported = false;

  double *plane_mem[2] = {nullptr, nullptr};
  Planes cur{}, alt{};
  long long *id_cur = nullptr, *id_alt = nullptr;
  int *fl_cur = nullptr, *fl_alt = nullptr;   // flume of every slot
  int *flume_of_id = nullptr;                  // flume of every clump id
  NbrRec *nbr = nullptr;
  CullRec *cull = nullptr;
  NbrRec *nbr_next = nullptr;     // the look-ahead's records of the next step
  CullRec *cull_next = nullptr;
  // The previous force pass ran this step's predictor (look-ahead): the step's predicted state is
  // in nbr/cull (records), the RN planes (rotation rows) and the cell keys; the planes still hold
  // the last step's corrected state.
  bool look = false;
  ContactLists lists{};   // the item lists of the current force pass
  Cells cells{};
  DevScalars *d = nullptr;
  DevFlume *flumes = nullptr;
  bool records_valid = false;   // records reflect the current planes
  bool cells_valid = false;     // start[] describes the current layout
  bool sorted = false;          // the slots are in the (cell, id) order of the last sort
  long resort_every = kResortEvery;   // steps between permutations = steps per long graph
  long since_sort = kResortEvery;   // steps since the planes were last permuted

  af3d_particle *d_aos = nullptr;
  double *d_acc = nullptr, *d_anga = nullptr;
  long long *d_tmp = nullptr;
  unsigned long long *d_count = nullptr;

  StepGraph graphs[4];
  int graph_next = 0;
  // af3d_step_host: the stream of its device-to-host copies and the events that release them
  cudaStream_t xfer = nullptr;
  cudaEvent_t part_done[kHostParts] = {}, part_in[kHostParts] = {};
  long launches = 0;          // kernels executed (graph replays included)

  Launch L() const { return Launch{st, n}; }
};

namespace {

void swap_accel_planes(Planes &P) {
  for (int k = 0; k < 6; k++) std::swap(P.p[AIX + k], P.p[AFX + k]);
}

void swap_velocity_planes(Planes &a, Planes &b) {
  for (int k = 0; k < 6; k++) std::swap(a.p[VX + k], b.p[VX + k]);
}

bool same_planes(const Planes &a, const Planes &b) {
  return std::memcmp(&a, &b, sizeof(Planes)) == 0;
}

PtrState ptr_state(const af3d_ctx *c) {
  return PtrState{c->cur, c->alt, c->id_cur, c->id_alt, c->fl_cur, c->fl_alt, c->nbr, c->nbr_next, c->cull,
                  c->cull_next, c->look};
}

void set_ptr_state(af3d_ctx *c, const PtrState &p) {
  c->cur = p.cur; c->alt = p.alt;
  c->id_cur = p.id_cur; c->id_alt = p.id_alt;
  c->fl_cur = p.fl_cur; c->fl_alt = p.fl_alt;
  c->nbr = p.nbr; c->nbr_next = p.nbr_next;
  c->cull = p.cull; c->cull_next = p.cull_next;
  c->look = p.look;
}

bool same_state(const PtrState &a, const PtrState &b) {
  return same_planes(a.cur, b.cur) && same_planes(a.alt, b.alt) && a.id_cur == b.id_cur &&
         a.id_alt == b.id_alt && a.fl_cur == b.fl_cur && a.fl_alt == b.fl_alt && a.nbr == b.nbr &&
         a.nbr_next == b.nbr_next && a.cull == b.cull && a.cull_next == b.cull_next && a.look == b.look;
}

void drop_graphs(af3d_ctx *c) {
  for (auto &g : c->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = StepGraph{};
  }
}

// Host-side parameter edits (system_par, Funnel, clock, phase, friction) to the device; the
// device-derived grids are read back first so that they are not overwritten.
af3d_status push_params(af3d_ctx *c) {
  drop_graphs(c);   // graphs hold the constants of their force launches
  std::vector<DevFlume> fl(c->nflumes);
  AF3D_CUDA(cudaMemcpyAsync(fl.data(), c->flumes, sizeof(DevFlume) * c->nflumes, cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  for (int f = 0; f < c->nflumes; f++) {
    fl[f].sys = c->sys[f];
    fl[f].sys.time = c->time;
    fl[f].fun = c->fun[f];
    fl[f].tant = c->sys[f].sint / c->sys[f].cost;
    fl[f].c = make_consts(c->sys[f], c->fun[f], fl[f].tant, c->phase, c->variant, &c->d->time);
  }
  AF3D_CUDA(cudaMemcpyAsync(c->flumes, fl.data(), sizeof(DevFlume) * c->nflumes, cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaMemcpyAsync(&c->d->time, &c->time, sizeof(double), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaMemcpyAsync(&c->d->phase, &c->phase, sizeof(int), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaMemcpyAsync(&c->d->variant, &c->variant, sizeof(int), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  return AF3D_OK;
}

af3d_status pull_params(af3d_ctx *c) {
  std::vector<DevFlume> fl(c->nflumes);
  AF3D_CUDA(cudaMemcpyAsync(fl.data(), c->flumes, sizeof(DevFlume) * c->nflumes, cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaMemcpyAsync(&c->time, &c->d->time, sizeof(double), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  for (int f = 0; f < c->nflumes; f++) c->grid[f] = fl[f].grid;
  return AF3D_OK;
}

af3d_status ensure_buckets(af3d_ctx *c, long ncell_total) {
  const long need = ncell_total + c->n + 1;
  if (need <= c->cells.cap && c->cells.count) return AF3D_OK;
  const long cap = std::max<long>(need + need / 2, 1024);
  if (cap > (1L << 31) - 2) return fail(AF3D_ERR_NOMEM, "cell grid too large for 32-bit bucket indices");
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  cudaFree(c->cells.count);
  cudaFree(c->cells.start);
  cudaFree(c->cells.tile_count);
  c->cells.count = c->cells.start = c->cells.tile_count = nullptr;
  AF3D_CUDA(cudaMalloc(&c->cells.count, sizeof(int) * cap));
  AF3D_CUDA(cudaMalloc(&c->cells.start, sizeof(int) * (cap + 1)));
  AF3D_CUDA(cudaMalloc(&c->cells.tile_count, sizeof(int) * (scan_tiles(cap) + 1)));
  AF3D_CUDA(cudaMemsetAsync(c->cells.count, 0, sizeof(int) * cap, c->st));
  AF3D_CUDA(cudaMemsetAsync(c->cells.tile_count, 0, sizeof(int) * (scan_tiles(cap) + 1), c->st));
  c->cells.cap = cap;
  c->cells_valid = false;
  drop_graphs(c);
  return AF3D_OK;
}

// Install host grids for every flume (cell offsets in flume order).
af3d_status set_grids_device(af3d_ctx *c) {
  long long total = 0;
  for (int f = 0; f < c->nflumes; f++) total += c->grid[f].ncell3;
  af3d_status s = ensure_buckets(c, total);
  if (s) return s;
  std::vector<DevFlume> fl(c->nflumes);
  AF3D_CUDA(cudaMemcpyAsync(fl.data(), c->flumes, sizeof(DevFlume) * c->nflumes, cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  long long off = 0;
  for (int f = 0; f < c->nflumes; f++) {
    fl[f].grid = c->grid[f];
    fl[f].gridf = grid_floats(c->grid[f]);
    fl[f].cell_off = off;
    off += c->grid[f].ncell3;
  }
  AF3D_CUDA(cudaMemcpyAsync(c->flumes, fl.data(), sizeof(DevFlume) * c->nflumes, cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaMemcpyAsync(&c->d->ncell_total, &total, sizeof(long long), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  c->have_grid = true;
  c->cells_valid = false;
  return AF3D_OK;
}

// Device re-grid of every flume, then adopt the result on the host (grow the bucket buffers and
// commit again if the new grids did not fit).
af3d_status regrid(af3d_ctx *c) {
  if (c->n == 0) return AF3D_OK;   // no clump to bound (cell_dim reads pp[0]): keep the grids
  launch_regrid(c->L(), c->cur, c->d, c->fl_cur, c->nflumes, c->cells.cap);
  c->launches += kKernelsPerRegrid;
  long long pending = 0;
  AF3D_CUDA(cudaMemcpyAsync(&pending, &c->d->pending, sizeof(long long), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  if (pending < 0) return fail(AF3D_ERR_GRID_ESCAPE, "re-grid produced an empty grid");
  if (pending > 0) {
    af3d_status s = ensure_buckets(c, pending);
    if (s) return s;
    launch_commit_grids(c->st, c->d, c->nflumes, c->n, c->cells.cap);
    AF3D_CUDA(cudaMemcpyAsync(&pending, &c->d->pending, sizeof(long long), cudaMemcpyDeviceToHost, c->st));
    AF3D_CUDA(cudaStreamSynchronize(c->st));
    if (pending != 0) return fail(AF3D_ERR_NOMEM, "re-grid does not fit after growing the buckets");
  }
  c->have_grid = true;
  c->cells_valid = false;
  return pull_params(c);
}

// clear_cell + clear_ocup + cell_locate: keys (optionally fused with the predictor), counting
// sort, permutation of every plane into the new order, neighbour records.
// The predictor and force launchers of the context's FP64 mode (the other kernels have one form).
void predict_for(af3d_ctx *c, bool predict, bool keys, bool t_prev, bool records = false, long s0 = 0,
                 long count = -1) {
  NbrRec *nbr = records ? c->nbr : nullptr;
  CullRec *cull = records ? c->cull : nullptr;
  if (c->fp_mode == AF3D_FP_FAST)
    fast::launch_predict(c->L(), c->cur, c->d, predict, keys, t_prev, c->cells, c->id_cur, c->fl_cur, nbr, cull,
                         s0, count);
  else
    launch_predict(c->L(), c->cur, c->d, predict, keys, t_prev, c->cells, c->id_cur, c->fl_cur, nbr, cull, s0,
                   count);
}

// order: null when the slots were just permuted into (cell, id) order; out: where the corrected
// velocities go.
// A single-flume context passes its constants as a kernel parameter (from the host mirrors,
// which push_params keeps equal to the device table; captured graphs are dropped whenever they
// change).
void forces_for(af3d_ctx *c, bool write_ft, const int *order, Planes out, bool warm = false, bool look = false,
                long s0 = 0, long count = -1) {
  const float4 *csort = order ? c->cells.csort : nullptr;
  Consts kc;
  const Consts *uni = nullptr;
  if (c->nflumes == 1) {
    kc = make_consts(c->sys[0], c->fun[0], c->sys[0].sint / c->sys[0].cost, c->phase, c->variant, &c->d->time);
    uni = &kc;
  }
  LookAhead la{};
  if (look) la = LookAhead{c->nbr_next, c->cull_next, c->cells, c->id_cur};
  if (c->fp_mode == AF3D_FP_FAST)
    fast::launch_lists_forces(c->L(), c->cur, out, c->d, c->fl_cur, c->nbr, c->cull, c->cells.start, order, csort,
                              c->lists, write_ft, uni, warm, la, s0, count, c->force_shape);
  else
    launch_lists_forces(c->L(), c->cur, out, c->d, c->fl_cur, c->nbr, c->cull, c->cells.start, order, csort,
                        c->lists, write_ft, uni, warm, la, s0, count, c->force_shape);
}

void enqueue_cell_build(af3d_ctx *c, bool predict, bool t_prev, bool ft = true) {
  predict_for(c, predict, true, t_prev);
  launch_sort(c->L(), c->d, c->cells, c->id_cur, c->ntags);
  launch_permute_records(c->L(), c->cur, c->alt, c->cells.perm, c->id_cur, c->id_alt, c->fl_cur, c->fl_alt,
                         c->nbr, c->cull, ft);
  std::swap(c->cur, c->alt);
  std::swap(c->id_cur, c->id_alt);
  std::swap(c->fl_cur, c->fl_alt);
  c->sorted = true;
  c->since_sort = 0;
}

// One fused step: time += dt, init_Verlet + cell build, every force of the phase, get_accel,
// finish_Verlet, and the acceleration swap.  With `resort` the planes are permuted into the new
// (cell, id) order; otherwise the predictor writes the records at the clumps' own slots, the
// force pass reaches the sorted order through cells.perm and corrects the velocities in place.
// When the previous pass looked ahead (c->look), this step's predictor has already run and the
// step is the sort and the force pass.  `look`: this step's force pass runs the next step's
// predictor.
void enqueue_fused_step(af3d_ctx *c, bool resort, bool write_ft = false, bool look = false) {
  const bool warm = !resort && c->look;
  if (!warm) launch_advance_time(c->st, c->d);   // a warm step advances the clock in its sort
  if (resort) {
    enqueue_cell_build(c, true, true, false);   // F, T and a_f are rewritten before being read
    forces_for(c, write_ft, nullptr, c->alt, false, look);
    swap_velocity_planes(c->cur, c->alt);
  } else {
    if (!warm) predict_for(c, true, true, true, true);
    launch_sort(c->L(), c->d, c->cells, c->id_cur, c->ntags, c->cull, warm);
    forces_for(c, write_ft, c->cells.perm, c->cur, warm, look);
  }
  if (look) {
    std::swap(c->nbr, c->nbr_next);
    std::swap(c->cull, c->cull_next);
  }
  c->look = look;
  swap_accel_planes(c->cur);
  swap_accel_planes(c->alt);
  c->sorted = resort;
}

// Kernels of `len` fused steps, the first one permuting (resort_first) or, with look_first,
// predicted by the previous pass; every later step is predicted by its previous pass.
long kernels_of(long len, bool resort_first, bool look_first) {
  // a predicted step skips the predictor and advances the clock inside its sort
  const long warm = kKernelsPerKeptStep - 2;
  const long first = resort_first ? kKernelsPerStep : (look_first ? warm : kKernelsPerKeptStep);
  return first + (len - 1) * warm;
}

// launch false: capture (and cache) the graphs m steps would replay without running anything;
// the caller restores the context's step state afterwards.
af3d_status run_steps(af3d_ctx *c, long m, bool launch = true) {
  // Captured graphs of resort_every steps (the first one permuting the planes) while that many
  // steps remain, then of two steps (permuting first only when the last permutation is due); an odd
  // last step is enqueued directly.  A graph is replayed when the context is in the pointer
  // state it was captured from, and leaves the context in the state it ended in.  A force pass
  // looks ahead (runs the next step's predictor) when the next step of the run keeps the slot
  // order; a permuting step predicts from the planes itself.
  auto resorts = [&](long since, long left) {   // does the next batch of `left` steps permute first?
    if (left >= 2) {
      const long l = left >= c->resort_every ? c->resort_every : 2;
      return l == c->resort_every || since + l > c->resort_every;
    }
    return since + 1 > c->resort_every;
  };
  while (m >= 2) {
    const long len = m >= c->resort_every ? c->resort_every : 2;
    const bool resort_first = len == c->resort_every || c->since_sort + len > c->resort_every;
    const long since_after = resort_first ? len - 1 : c->since_sort + len;
    const bool look_last = m > len && !resorts(since_after, m - len);
    const bool look_first = c->look;
    const PtrState now = ptr_state(c);
    StepGraph *g = nullptr;
    for (auto &cand : c->graphs)
      if (cand.exec && cand.steps == len && cand.resort_first == resort_first && cand.look_last == look_last &&
          same_state(cand.start, now))
        g = &cand;
    if (!g) {
      g = &c->graphs[c->graph_next];
      c->graph_next = (c->graph_next + 1) % 4;
      if (g->exec) cudaGraphExecDestroy(g->exec);
      *g = StepGraph{};
      g->start = now;
      g->steps = len;
      g->resort_first = resort_first;
      g->look_last = look_last;
      cudaGraph_t graph;
      AF3D_CUDA(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
      for (long i = 0; i < len; i++) enqueue_fused_step(c, i == 0 && resort_first, false, i + 1 < len || look_last);
      AF3D_CUDA(cudaStreamEndCapture(c->st, &graph));
      g->end = ptr_state(c);
      set_ptr_state(c, now);
      cudaError_t e = cudaGraphInstantiate(&g->exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) {
        g->exec = nullptr;
        return fail(AF3D_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
      }
    }
    if (launch) AF3D_CUDA(cudaGraphLaunch(g->exec, c->st));
    set_ptr_state(c, g->end);
    c->sorted = false;   // the last captured step keeps the slot order
    c->since_sort = since_after;
    if (launch) c->launches += kernels_of(len, resort_first, look_first);
    m -= len;
  }
  if (m == 1 && launch) {
    const bool resort = c->since_sort + 1 > c->resort_every;
    const bool look_first = c->look;
    enqueue_fused_step(c, resort);
    c->since_sort = resort ? 0 : c->since_sort + 1;
    c->launches += kernels_of(1, resort, look_first);
  }
  return AF3D_OK;
}

af3d_status read_status(af3d_ctx *c, int *flags) {
  int st = 0, zero = 0;
  AF3D_CUDA(cudaMemcpyAsync(&st, &c->d->status, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaMemcpyAsync(&c->d->status, &zero, sizeof(int), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  AF3D_CUDA(cudaGetLastError());
  *flags = st;
  return AF3D_OK;
}

af3d_status first_error(int flags) {
  for (int e : {AF3D_ERR_NAN, AF3D_ERR_NEGATIVE_CELL, AF3D_ERR_GRID_ESCAPE, AF3D_ERR_CELL_CAPACITY})
    if (flags & (1 << e)) return fail(e, "device check raised status bit " + std::to_string(e));
  return AF3D_OK;
}

af3d_status ensure_records(af3d_ctx *c) {
  if (!c->imported) return fail(AF3D_ERR_ARG, "no particles imported");
  if (!c->cells_valid) return fail(AF3D_ERR_ARG, "no cell build since the last grid change");
  if (!c->sorted) return fail(AF3D_ERR_ARG, "af3d_step left the slots out of cell order: call af3d_cell_build");
  if (!c->records_valid) {
    launch_build_records(c->L(), c->cur, c->nbr, c->cull);
    c->records_valid = true;
  }
  return AF3D_OK;
}

// Plane-resident per-clump vectors back to clump-id order on the host.
af3d_status gather_by_id(af3d_ctx *c, int plane0, af3d_vec3 *a, af3d_vec3 *b) {
  if (c->n == 0) return AF3D_OK;
  std::vector<double> hp(6 * (size_t)c->n);
  std::vector<long long> ids((size_t)c->n);
  for (int k = 0; k < 6; k++)
    AF3D_CUDA(cudaMemcpyAsync(hp.data() + (size_t)k * c->n, c->cur.p[plane0 + k], sizeof(double) * c->n,
                              cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaMemcpyAsync(ids.data(), c->id_cur, sizeof(long long) * c->n, cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  for (long s = 0; s < c->n; s++) {
    const long long i = ids[s];
    if (a) a[i] = {hp[s], hp[c->n + s], hp[2 * c->n + s]};
    if (b) b[i] = {hp[3 * c->n + s], hp[4 * c->n + s], hp[5 * c->n + s]};
  }
  return AF3D_OK;
}

#define CHECK_CTX(c)                                                                            \
  do {                                                                                          \
    if (!(c)) return fail(AF3D_ERR_ARG, "null context");                                       \
  } while (0)
#define CHECK_STATE(c)                                                                          \
  do {                                                                                          \
    CHECK_CTX(c);                                                                               \
    if (!(c)->imported) return fail(AF3D_ERR_ARG, "no particles imported");                    \
  } while (0)
#define CHECK_FLUME(c, f)                                                                       \
  do {                                                                                          \
    if ((f) < 0 || (f) >= (c)->nflumes) return fail(AF3D_ERR_ARG, "flume index out of range");  \
  } while (0)

}  // namespace

extern "C" {

const char *af3d_last_error(void) { return g_last_error.c_str(); }
int af3d_abi_version(void) { return AF3D_ABI_VERSION; }

af3d_status af3d_create_ensemble(int nflumes, const af3d_system_par *sys, const af3d_funnel *fun,
                                 long ntags, int phase, af3d_ctx **out) {
  if (!sys || !fun || !out || nflumes < 1) return fail(AF3D_ERR_ARG, "bad argument");
  *out = nullptr;
  long total = 0;
  for (int f = 0; f < nflumes; f++) {
    if (sys[f].npart < 0) return fail(AF3D_ERR_ARG, "negative npart");
    if (sys[f].dt != sys[0].dt || sys[f].hdt != sys[0].hdt)
      return fail(AF3D_ERR_ARG, "the flumes of an ensemble share dt");
    total += sys[f].npart;
  }
  // Slots are packed with a 4-bit sphere-pair index into 32-bit work items, and the top 256
  // codes are reserved for boundary items: at most 2^28 - 16 clumps.
  if (total > (1L << 28) - 16) return fail(AF3D_ERR_ARG, "too many clumps (at most 2^28 - 16)");
  af3d_ctx *c = new af3d_ctx();
  c->n = total;
  c->nflumes = nflumes;
  c->sys.assign(sys, sys + nflumes);
  c->fun.assign(fun, fun + nflumes);
  c->grid.assign(nflumes, af3d_cell_par{});
  for (auto &g : c->grid) g.ntags = ntags;
  c->first_id.resize(nflumes + 1, 0);
  for (int f = 0; f < nflumes; f++) c->first_id[f + 1] = c->first_id[f] + sys[f].npart;
  c->time = sys[0].time;
  c->ntags = ntags;
  c->phase = phase;
  cudaError_t e = cudaGetDevice(&c->device);
  int sms = 0;
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
  c->force_shape = force_shape_for(c->n, sms);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return fail(AF3D_ERR_CUDA, std::string("CUDA unavailable: ") + cudaGetErrorString(e));
  }
  c->own_stream = true;
  const long n = std::max<long>(c->n, 1);
  bool ok = true;
  for (int b = 0; b < 2 && ok; b++)
    ok = cudaMalloc((void **)&c->plane_mem[b], sizeof(double) * n * NPLANES) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->id_cur, sizeof(long long) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->id_alt, sizeof(long long) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->fl_cur, sizeof(int) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->fl_alt, sizeof(int) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->flume_of_id, sizeof(int) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->nbr, sizeof(NbrRec) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->cull, sizeof(CullRec) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->nbr_next, sizeof(NbrRec) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->cull_next, sizeof(CullRec) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->lists.items, sizeof(unsigned) * kListCap * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->cells.key, sizeof(int) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->cells.rank_tmp, sizeof(int) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->cells.tmp_slot, sizeof(int) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->cells.perm, sizeof(int) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->cells.csort, sizeof(float4) * n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->d, sizeof(DevScalars)) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->flumes, sizeof(DevFlume) * nflumes) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&c->d_count, sizeof(unsigned long long)) == cudaSuccess;
  if (!ok) {
    af3d_destroy(c);
    return fail(AF3D_ERR_NOMEM, "device allocation failed");
  }
  for (int k = 0; k < NPLANES; k++) {
    c->cur.p[k] = c->plane_mem[0] + (size_t)k * n;
    c->alt.p[k] = c->plane_mem[1] + (size_t)k * n;
  }
  std::vector<int> fid((size_t)n, 0);
  for (int f = 0; f < nflumes; f++)
    for (long i = c->first_id[f]; i < c->first_id[f + 1]; i++) fid[i] = f;
  std::vector<DevFlume> fl(nflumes);
  std::memset(fl.data(), 0, sizeof(DevFlume) * nflumes);
  for (int f = 0; f < nflumes; f++) {
    fl[f].sys = c->sys[f];
    fl[f].fun = c->fun[f];
    fl[f].grid = c->grid[f];
    fl[f].gridf = grid_floats(c->grid[f]);
    fl[f].pending = c->grid[f];
    fl[f].tant = c->sys[f].sint / c->sys[f].cost;
    fl[f].c = make_consts(c->sys[f], c->fun[f], fl[f].tant, phase, c->variant, &c->d->time);
  }
  DevScalars ds;
  std::memset(&ds, 0, sizeof ds);
  ds.time = c->time;
  ds.time_prev = c->time;
  ds.phase = phase;
  ds.variant = c->variant;
  ds.nflumes = nflumes;
  ds.flumes = c->flumes;
  cudaMemsetAsync(c->plane_mem[0], 0, sizeof(double) * n * NPLANES, c->st);
  cudaMemsetAsync(c->plane_mem[1], 0, sizeof(double) * n * NPLANES, c->st);
  cudaMemcpyAsync(c->flume_of_id, fid.data(), sizeof(int) * n, cudaMemcpyHostToDevice, c->st);
  cudaMemcpyAsync(c->flumes, fl.data(), sizeof(DevFlume) * nflumes, cudaMemcpyHostToDevice, c->st);
  cudaMemcpyAsync(c->d, &ds, sizeof ds, cudaMemcpyHostToDevice, c->st);
  e = cudaStreamSynchronize(c->st);
  if (e != cudaSuccess) {
    af3d_destroy(c);
    return fail(AF3D_ERR_CUDA, std::string("context set-up: ") + cudaGetErrorString(e));
  }
  *out = c;
  return AF3D_OK;
}

af3d_status af3d_create(const af3d_system_par *sys, const af3d_funnel *fun, long ntags, int phase,
                        af3d_ctx **out) {
  return af3d_create_ensemble(1, sys, fun, ntags, phase, out);
}

af3d_status af3d_destroy(af3d_ctx *c) {
  if (!c) return AF3D_OK;
  if (c->st) cudaStreamSynchronize(c->st);
  drop_graphs(c);
  for (void *p : {(void *)c->plane_mem[0], (void *)c->plane_mem[1], (void *)c->id_cur, (void *)c->id_alt,
                  (void *)c->fl_cur, (void *)c->fl_alt, (void *)c->flume_of_id, (void *)c->nbr,
                  (void *)c->cull, (void *)c->lists.items, (void *)c->nbr_next, (void *)c->cull_next, (void *)c->cells.key, (void *)c->cells.rank_tmp, (void *)c->cells.tmp_slot,
                  (void *)c->cells.perm, (void *)c->cells.csort, (void *)c->cells.count, (void *)c->cells.start,
                  (void *)c->cells.tile_count, (void *)c->d, (void *)c->flumes, (void *)c->d_aos,
                  (void *)c->d_acc, (void *)c->d_anga, (void *)c->d_tmp, (void *)c->d_count})
    if (p) cudaFree(p);
  if (c->own_stream && c->st) cudaStreamDestroy(c->st);
  if (c->xfer) {
    cudaStreamSynchronize(c->xfer);
    cudaStreamDestroy(c->xfer);
  }
  for (cudaEvent_t e : c->part_done)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : c->part_in)
    if (e) cudaEventDestroy(e);
  delete c;
  return AF3D_OK;
}

af3d_status af3d_set_stream(af3d_ctx *c, void *stream) {
  CHECK_CTX(c);
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  if (c->own_stream) cudaStreamDestroy(c->st);
  drop_graphs(c);
  if (stream) {
    c->st = (cudaStream_t)stream;
    c->own_stream = false;
  } else {
    AF3D_CUDA(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
    c->own_stream = true;
  }
  return AF3D_OK;
}

af3d_status af3d_set_friction(af3d_ctx *c, int variant) {
  CHECK_CTX(c);
  if (variant != AF3D_FRICTION_HST && variant != AF3D_FRICTION_DEV)
    return fail(AF3D_ERR_ARG, "unknown friction variant");
  c->variant = variant;
  return push_params(c);
}

af3d_status af3d_set_objective(af3d_ctx *c, int objective, double length) {
  CHECK_CTX(c);
  if (objective == AF3D_OBJ_CENTROID) {
    c->obj_length = 0.0;
  } else if (objective == AF3D_OBJ_RUNOUT) {
    if (!(length > 0.0) || !std::isfinite(length)) return fail(AF3D_ERR_ARG, "the runout length scale must be > 0");
    c->obj_length = length;
  } else {
    return fail(AF3D_ERR_ARG, "unknown objective");
  }
  return AF3D_OK;
}

af3d_status af3d_set_fp_mode(af3d_ctx *c, int mode) {
  CHECK_CTX(c);
  if (mode != AF3D_FP_EXACT && mode != AF3D_FP_FAST) return fail(AF3D_ERR_ARG, "unknown FP64 mode");
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  if (mode != c->fp_mode) drop_graphs(c);
  c->fp_mode = mode;
  return AF3D_OK;
}

namespace {

// The host particle array (and accelerations) into the plane set, enqueued on the context's
// stream.  keep_order: every clump goes back to the slot it held; otherwise slot i receives
// clump i.
af3d_status enqueue_import(af3d_ctx *c, const af3d_particle *pp, const af3d_vec3 *acc, const af3d_vec3 *anga,
                           bool keep_order) {
  const long n = std::max<long>(c->n, 1);
  if (!c->d_aos) AF3D_CUDA(cudaMalloc(&c->d_aos, sizeof(af3d_particle) * n));
  if (!c->d_acc) AF3D_CUDA(cudaMalloc(&c->d_acc, sizeof(double) * 3 * n));
  if (!c->d_anga) AF3D_CUDA(cudaMalloc(&c->d_anga, sizeof(double) * 3 * n));
  if (c->n > 0) {
    AF3D_CUDA(cudaMemcpyAsync(c->d_aos, pp, sizeof(af3d_particle) * c->n, cudaMemcpyHostToDevice, c->st));
    if (acc) AF3D_CUDA(cudaMemcpyAsync(c->d_acc, acc, sizeof(double) * 3 * c->n, cudaMemcpyHostToDevice, c->st));
    if (anga) AF3D_CUDA(cudaMemcpyAsync(c->d_anga, anga, sizeof(double) * 3 * c->n, cudaMemcpyHostToDevice, c->st));
  }
  launch_aos_to_planes(c->L(), c->d_aos, acc ? c->d_acc : nullptr, anga ? c->d_anga : nullptr, c->flume_of_id,
                       c->cur, c->id_cur, c->fl_cur, keep_order);
  c->imported = true;
  c->records_valid = false;
  c->cells_valid = false;
  c->sorted = false;
  c->look = false;
  if (!keep_order) {
    c->since_sort = c->resort_every;
    drop_graphs(c);
  }
  return AF3D_OK;
}

}  // namespace

af3d_status af3d_import_particles(af3d_ctx *c, const af3d_particle *pp, const af3d_vec3 *acc,
                                  const af3d_vec3 *anga) {
  CHECK_CTX(c);
  if (!pp && c->n > 0) return fail(AF3D_ERR_ARG, "null particle array");
  // A re-import keeps the slot order of the last permutation (every clump stays in its slot),
  // so the next step need not permute; the first import puts clump i in slot i.
  af3d_status s = enqueue_import(c, pp, acc, anga, c->imported);
  if (s) return s;
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  AF3D_CUDA(cudaGetLastError());
  if (!c->have_grid && c->n > 0) return regrid(c);
  return AF3D_OK;
}

af3d_status af3d_export_particles(af3d_ctx *c, af3d_particle *pp, af3d_vec3 *acc, af3d_vec3 *anga) {
  CHECK_STATE(c);
  if (!pp && c->n > 0) return fail(AF3D_ERR_ARG, "null particle array");
  launch_planes_to_aos(c->L(), c->cur, c->id_cur, c->fl_cur, c->d_aos, acc ? c->d_acc : nullptr,
                       anga ? c->d_anga : nullptr, c->d);
  if (c->n > 0) {
    AF3D_CUDA(cudaMemcpyAsync(pp, c->d_aos, sizeof(af3d_particle) * c->n, cudaMemcpyDeviceToHost, c->st));
    if (acc) AF3D_CUDA(cudaMemcpyAsync(acc, c->d_acc, sizeof(double) * 3 * c->n, cudaMemcpyDeviceToHost, c->st));
    if (anga) AF3D_CUDA(cudaMemcpyAsync(anga, c->d_anga, sizeof(double) * 3 * c->n, cudaMemcpyDeviceToHost, c->st));
  }
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  AF3D_CUDA(cudaGetLastError());
  return AF3D_OK;
}

af3d_status af3d_step_host(af3d_ctx *c, const af3d_particle *in, const af3d_vec3 *acc_in,
                           const af3d_vec3 *anga_in, af3d_particle *out, af3d_vec3 *acc_out,
                           af3d_vec3 *anga_out) {
  CHECK_CTX(c);
  const long n = c->n;
  if (n > 0 && (!in || !out)) return fail(AF3D_ERR_ARG, "null particle array");
  if (!c->have_grid || n == 0) {
    // no grid yet (the import derives it) or nothing to overlap: the three calls in turn
    af3d_status s = af3d_import_particles(c, in, acc_in, anga_in);
    if (s) return s;
    s = af3d_step(c, 1);
    if (s) return s;
    return af3d_export_particles(c, out, acc_out, anga_out);
  }
  const long m = n;
  if (!c->d_aos) AF3D_CUDA(cudaMalloc(&c->d_aos, sizeof(af3d_particle) * m));
  if (!c->d_acc) AF3D_CUDA(cudaMalloc(&c->d_acc, sizeof(double) * 3 * m));
  if (!c->d_anga) AF3D_CUDA(cudaMalloc(&c->d_anga, sizeof(double) * 3 * m));
  if (!c->xfer) AF3D_CUDA(cudaStreamCreateWithFlags(&c->xfer, cudaStreamNonBlocking));
  for (cudaEvent_t &e : c->part_done)
    if (!e) AF3D_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  for (cudaEvent_t &e : c->part_in)
    if (!e) AF3D_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  // Part boundaries on whole blocks.  The first part to leave the device (force pass, then copy
  // out) and the last part to arrive (copy in, then conversion and predictor) are the ones
  // whose work nothing overlaps, so they get half a part's share of the clumps and the others
  // share the rest: `out_at` splits the export, `in_at` (the mirror image) the import.
  auto round_up = [](long x) { return (x + kForceAlign - 1) / kForceAlign * kForceAlign; };
  const long edge = (n + 2 * kHostParts - 1) / (2 * kHostParts);
  long out_at[kHostParts + 1], in_at[kHostParts + 1];
  out_at[0] = 0;
  out_at[1] = std::min(n, round_up(edge));
  for (int j = 2; j <= kHostParts; j++)
    out_at[j] = std::min(n, out_at[1] + round_up((n - out_at[1]) * (j - 1) / (kHostParts - 1)));
  out_at[kHostParts] = n;
  in_at[0] = 0;
  for (int j = 1; j < kHostParts; j++) in_at[j] = std::min(n, round_up((n - edge) * j / (kHostParts - 1)));
  in_at[kHostParts] = n;
  // Import in input order (slot i holds clump i), so a part of the slots is a contiguous part of
  // the host arrays; the step keeps that order (the cell sort only orders the neighbour search).
  // Each part's copy to the device (copy stream) releases its conversion to planes and its
  // predictor (the step's stream) while the next part copies.  The copy stream waits for the
  // context's stream first: the staging buffers may still be in use.
  AF3D_CUDA(cudaEventRecord(c->part_done[0], c->st));
  AF3D_CUDA(cudaStreamWaitEvent(c->xfer, c->part_done[0], 0));
  drop_graphs(c);   // the slot order changes (the next af3d_step permutes when it is due)
  launch_advance_time(c->st, c->d);
  int parts = 0;
  for (int j = 0; j < kHostParts; j++) {
    const long s0 = in_at[j], cnt = in_at[j + 1] - s0;
    if (cnt <= 0) continue;
    AF3D_CUDA(cudaMemcpyAsync(c->d_aos + s0, in + s0, sizeof(af3d_particle) * cnt, cudaMemcpyHostToDevice,
                              c->xfer));
    if (acc_in)
      AF3D_CUDA(cudaMemcpyAsync(c->d_acc + 3 * s0, acc_in + s0, sizeof(double) * 3 * cnt, cudaMemcpyHostToDevice,
                                c->xfer));
    if (anga_in)
      AF3D_CUDA(cudaMemcpyAsync(c->d_anga + 3 * s0, anga_in + s0, sizeof(double) * 3 * cnt,
                                cudaMemcpyHostToDevice, c->xfer));
    AF3D_CUDA(cudaEventRecord(c->part_in[parts], c->xfer));
    AF3D_CUDA(cudaStreamWaitEvent(c->st, c->part_in[parts], 0));
    launch_aos_to_planes(c->L(), c->d_aos, acc_in ? c->d_acc : nullptr, anga_in ? c->d_anga : nullptr,
                         c->flume_of_id, c->cur, c->id_cur, c->fl_cur, false, s0, cnt);
    predict_for(c, true, true, true, true, s0, cnt);
    parts++;
  }
  c->imported = true;
  c->records_valid = false;
  c->cells_valid = false;
  c->sorted = false;
  c->look = false;
  c->since_sort = c->resort_every;
  // The rest of the step (a kept-order step of af3d_step): the sort, then the force pass in
  // kHostParts launches of whole blocks; after each, the part's clumps go to the AoS staging
  // buffer and, on the copy stream, to the host while the next part computes.
  launch_sort(c->L(), c->d, c->cells, c->id_cur, c->ntags, c->cull, false);
  Planes after = c->cur;   // the plane set as the step leaves it (accelerations swapped)
  swap_accel_planes(after);
  const int in_parts = parts;
  parts = 0;
  for (int j = 0; j < kHostParts; j++) {
    const long s0 = out_at[j], cnt = out_at[j + 1] - s0;
    if (cnt <= 0) continue;
    forces_for(c, false, c->cells.perm, c->cur, false, false, s0, cnt);
    launch_planes_to_aos(c->L(), after, c->id_cur, c->fl_cur, c->d_aos, acc_out ? c->d_acc : nullptr,
                         anga_out ? c->d_anga : nullptr, c->d, s0, cnt);
    AF3D_CUDA(cudaEventRecord(c->part_done[parts], c->st));
    AF3D_CUDA(cudaStreamWaitEvent(c->xfer, c->part_done[parts], 0));
    AF3D_CUDA(cudaMemcpyAsync(out + s0, c->d_aos + s0, sizeof(af3d_particle) * cnt, cudaMemcpyDeviceToHost,
                              c->xfer));
    if (acc_out)
      AF3D_CUDA(cudaMemcpyAsync(acc_out + s0, c->d_acc + 3 * s0, sizeof(double) * 3 * cnt, cudaMemcpyDeviceToHost,
                                c->xfer));
    if (anga_out)
      AF3D_CUDA(cudaMemcpyAsync(anga_out + s0, c->d_anga + 3 * s0, sizeof(double) * 3 * cnt,
                                cudaMemcpyDeviceToHost, c->xfer));
    parts++;
  }
  swap_accel_planes(c->cur);
  swap_accel_planes(c->alt);
  c->launches += (kKernelsPerKeptStep - kKernelsPerForcePass - 1) + 2L * in_parts + 2L * parts;
  // af3d_step's bookkeeping for one step
  c->time = c->time + c->sys[0].dt;
  const bool do_regrid = c->cc % kRegridEvery == 0;
  c->cc += 1;
  c->cells_valid = true;
  c->records_valid = false;
  AF3D_CUDA(cudaStreamSynchronize(c->xfer));
  af3d_status s = AF3D_OK;
  if (do_regrid) {
    s = regrid(c);
    if (s) return s;
  }
  int flags = 0;
  s = read_status(c, &flags);
  if (s) return s;
  return first_error(flags);
}

namespace {

// Lossless checkpoint file: this header, then per flume its system_par, Funnel and cell_par,
// then the particles (AoS, id order), a_i and alpha_i, all as raw host bytes.
struct CheckpointHeader {
  char magic[8];       // "AF3DCKP1"
  uint32_t layout;     // sizeof of particle, system_par, cell_par packed (a layout check)
  int32_t nflumes;
  int64_t n, ntags, cc;
  int32_t phase, variant, fp_mode, have_grid;
  double time;
};
constexpr char kCheckpointMagic[8] = {'A', 'F', '3', 'D', 'C', 'K', 'P', '1'};
constexpr uint32_t kCheckpointLayout =
    (uint32_t)sizeof(af3d_particle) | (uint32_t)sizeof(af3d_system_par) << 10 | (uint32_t)sizeof(af3d_cell_par) << 20;

}  // namespace

af3d_status af3d_save_checkpoint(af3d_ctx *c, const char *path) {
  CHECK_STATE(c);
  if (!path) return fail(AF3D_ERR_ARG, "null path");
  af3d_status s = pull_params(c);
  if (s) return s;
  const long n = c->n;
  std::vector<af3d_particle> pp((size_t)n);
  std::vector<af3d_vec3> a((size_t)n), al((size_t)n);
  s = af3d_export_particles(c, pp.data(), a.data(), al.data());
  if (s) return s;
  CheckpointHeader h{};
  std::memcpy(h.magic, kCheckpointMagic, 8);
  h.layout = kCheckpointLayout;
  h.nflumes = c->nflumes;
  h.n = n;
  h.ntags = c->ntags;
  h.cc = c->cc;
  h.phase = c->phase;
  h.variant = c->variant;
  h.fp_mode = c->fp_mode;
  h.have_grid = c->have_grid ? 1 : 0;
  h.time = c->time;
  FILE *fp = fopen(path, "wb");
  if (!fp) return fail(AF3D_ERR_IO, std::string("cannot write ") + path);
  bool ok = fwrite(&h, sizeof h, 1, fp) == 1;
  for (int f = 0; f < c->nflumes && ok; f++) {
    af3d_system_par sy = c->sys[f];
    sy.time = c->time;
    ok = fwrite(&sy, sizeof sy, 1, fp) == 1 && fwrite(&c->fun[f], sizeof(af3d_funnel), 1, fp) == 1 &&
         fwrite(&c->grid[f], sizeof(af3d_cell_par), 1, fp) == 1;
  }
  if (ok && n > 0)
    ok = fwrite(pp.data(), sizeof(af3d_particle), (size_t)n, fp) == (size_t)n &&
         fwrite(a.data(), sizeof(af3d_vec3), (size_t)n, fp) == (size_t)n &&
         fwrite(al.data(), sizeof(af3d_vec3), (size_t)n, fp) == (size_t)n;
  ok = (fclose(fp) == 0) && ok;
  return ok ? AF3D_OK : fail(AF3D_ERR_IO, std::string("write failed: ") + path);
}

af3d_status af3d_load_checkpoint(af3d_ctx *c, const char *path) {
  CHECK_CTX(c);
  if (!path) return fail(AF3D_ERR_ARG, "null path");
  FILE *fp = fopen(path, "rb");
  if (!fp) return fail(AF3D_ERR_IO, std::string("cannot read ") + path);
  CheckpointHeader h{};
  bool ok = fread(&h, sizeof h, 1, fp) == 1 && std::memcmp(h.magic, kCheckpointMagic, 8) == 0 &&
            h.layout == kCheckpointLayout;
  if (ok && (h.n != c->n || h.nflumes != c->nflumes || h.ntags != c->ntags)) {
    fclose(fp);
    return fail(AF3D_ERR_ARG, "checkpoint of another context shape (clumps, flumes or ntags differ)");
  }
  std::vector<af3d_system_par> sys(ok ? (size_t)h.nflumes : 0);
  std::vector<af3d_funnel> fun(sys.size());
  std::vector<af3d_cell_par> grid(sys.size());
  for (size_t f = 0; f < sys.size() && ok; f++)
    ok = fread(&sys[f], sizeof(af3d_system_par), 1, fp) == 1 && fread(&fun[f], sizeof(af3d_funnel), 1, fp) == 1 &&
         fread(&grid[f], sizeof(af3d_cell_par), 1, fp) == 1;
  const size_t n = ok ? (size_t)h.n : 0;
  std::vector<af3d_particle> pp(n);
  std::vector<af3d_vec3> a(n), al(n);
  if (ok && n > 0)
    ok = fread(pp.data(), sizeof(af3d_particle), n, fp) == n && fread(a.data(), sizeof(af3d_vec3), n, fp) == n &&
         fread(al.data(), sizeof(af3d_vec3), n, fp) == n;
  fclose(fp);
  if (!ok) return fail(AF3D_ERR_IO, std::string("not a readable checkpoint: ") + path);
  // parameters, clock, phase and modes; then the state; then the grids and the step counter
  af3d_status s = pull_params(c);
  if (s) return s;
  for (int f = 0; f < c->nflumes; f++) {
    c->sys[f] = sys[f];
    c->fun[f] = fun[f];
  }
  c->time = h.time;
  c->phase = h.phase;
  c->variant = h.variant;
  s = push_params(c);
  if (s) return s;
  s = af3d_set_fp_mode(c, h.fp_mode);
  if (s) return s;
  s = af3d_import_particles(c, pp.data(), a.data(), al.data());
  if (s) return s;
  if (h.have_grid)
    for (int f = 0; f < c->nflumes; f++) {
      s = af3d_set_flume_grid(c, f, &grid[f]);
      if (s) return s;
    }
  c->cc = h.cc;
  return AF3D_OK;
}

af3d_status af3d_set_flume_system(af3d_ctx *c, int f, const af3d_system_par *sys, const af3d_funnel *fun) {
  CHECK_CTX(c);
  CHECK_FLUME(c, f);
  if (!sys || sys->npart != c->first_id[f + 1] - c->first_id[f])
    return fail(AF3D_ERR_ARG, "system_par npart differs from the flume's");
  if (sys->dt != c->sys[0].dt && c->nflumes > 1) return fail(AF3D_ERR_ARG, "the flumes share dt");
  af3d_status s = pull_params(c);
  if (s) return s;
  c->sys[f] = *sys;
  if (fun) c->fun[f] = *fun;
  c->time = sys->time;
  return push_params(c);
}

af3d_status af3d_set_system(af3d_ctx *c, const af3d_system_par *sys) {
  CHECK_CTX(c);
  return af3d_set_flume_system(c, 0, sys, nullptr);
}

af3d_status af3d_get_flume_system(af3d_ctx *c, int f, af3d_system_par *sys) {
  CHECK_CTX(c);
  CHECK_FLUME(c, f);
  if (!sys) return fail(AF3D_ERR_ARG, "null argument");
  af3d_status s = pull_params(c);
  if (s) return s;
  *sys = c->sys[f];
  sys->time = c->time;
  return AF3D_OK;
}

af3d_status af3d_get_system(af3d_ctx *c, af3d_system_par *sys) { return af3d_get_flume_system(c, 0, sys); }

af3d_status af3d_set_flume_grid(af3d_ctx *c, int f, const af3d_cell_par *g) {
  CHECK_CTX(c);
  CHECK_FLUME(c, f);
  if (!g || g->ncell.x <= 0 || g->ncell.y <= 0 || g->ncell.z <= 0 ||
      g->ncell3 != g->ncell.x * g->ncell.y * g->ncell.z)
    return fail(AF3D_ERR_ARG, "inconsistent cell_par");
  if (c->have_grid) {
    af3d_status s = pull_params(c);
    if (s) return s;
  } else {
    for (auto &gg : c->grid)   // other flumes get a copy until they are set or re-gridded
      if (gg.ncell3 <= 0) gg = *g;
  }
  c->grid[f] = *g;
  c->grid[f].ntags = c->ntags;
  c->grid[f].ntot = c->grid[f].ncell3 * c->ntags;
  return set_grids_device(c);
}

af3d_status af3d_set_grid(af3d_ctx *c, const af3d_cell_par *g) { return af3d_set_flume_grid(c, 0, g); }

af3d_status af3d_get_flume_grid(af3d_ctx *c, int f, af3d_cell_par *g) {
  CHECK_CTX(c);
  CHECK_FLUME(c, f);
  if (!g) return fail(AF3D_ERR_ARG, "null argument");
  af3d_status s = pull_params(c);
  if (s) return s;
  *g = c->grid[f];
  return AF3D_OK;
}

af3d_status af3d_get_grid(af3d_ctx *c, af3d_cell_par *g) { return af3d_get_flume_grid(c, 0, g); }

int af3d_flume_count(af3d_ctx *c) { return c ? c->nflumes : 0; }

af3d_status af3d_set_phase(af3d_ctx *c, int phase) {
  CHECK_CTX(c);
  if (phase != AF3D_PHASE_FILL && phase != AF3D_PHASE_AVALANCHE) return fail(AF3D_ERR_ARG, "bad phase");
  af3d_status s = pull_params(c);
  if (s) return s;
  c->phase = phase;
  c->cc = 0;
  return push_params(c);
}

af3d_status af3d_regrid(af3d_ctx *c) {
  CHECK_STATE(c);
  return regrid(c);
}

af3d_status af3d_open_door(af3d_ctx *c) {
  CHECK_CTX(c);
  af3d_status s = pull_params(c);
  if (s) return s;
  for (auto &sy : c->sys) sy.side.x = (70.0 + sy.Lflume) * sy.cost;   // xfinal, avalanche_hst.cu:116
  c->time = 0.0;
  c->phase = AF3D_PHASE_AVALANCHE;
  c->cc = 0;
  return push_params(c);
}

// ---- per-routine entry points ----

af3d_status af3d_init_verlet(af3d_ctx *c) {
  CHECK_STATE(c);
  launch_predict(c->L(), c->cur, c->d, true, false, false, c->cells, c->id_cur, c->fl_cur);
  c->launches++;
  c->records_valid = false;
  return AF3D_OK;
}

af3d_status af3d_advance_time(af3d_ctx *c) {
  CHECK_CTX(c);
  launch_advance_time(c->st, c->d);
  c->launches++;
  c->time = c->time + c->sys[0].dt;
  return AF3D_OK;
}

af3d_status af3d_rotate_vectors(af3d_ctx *c) {
  // The slope-frame copies are recomputed by every routine that reads them (and by export), so
  // there is nothing to store.
  CHECK_STATE(c);
  return AF3D_OK;
}

af3d_status af3d_clear_forces(af3d_ctx *c) {
  CHECK_STATE(c);
  launch_clear_forces(c->L(), c->cur);
  c->launches++;
  return AF3D_OK;
}

af3d_status af3d_cell_build(af3d_ctx *c) {
  CHECK_STATE(c);
  if (!c->have_grid) return fail(AF3D_ERR_ARG, "no grid");
  enqueue_cell_build(c, false, false);
  c->launches += kKernelsPerCellBuild;
  c->records_valid = true;
  c->cells_valid = true;
  return AF3D_OK;
}

static af3d_status boundary(af3d_ctx *c, int routine) {
  CHECK_STATE(c);
  launch_boundary(c->L(), c->cur, c->d, c->fl_cur, routine);
  c->launches++;
  return AF3D_OK;
}

af3d_status af3d_force_hop(af3d_ctx *c, int nw) {
  CHECK_CTX(c);
  if (nw < 0 || nw > 2) return fail(AF3D_ERR_ARG, "nw must be 0, 1 or 2");
  return boundary(c, R_HOP0 + nw);
}
af3d_status af3d_force_funnel(af3d_ctx *c) { return boundary(c, R_FUNNEL); }
af3d_status af3d_force_fcorners(af3d_ctx *c) { return boundary(c, R_FCORNERS); }
af3d_status af3d_force_walls(af3d_ctx *c) { return boundary(c, R_WALLS); }
af3d_status af3d_force_flume(af3d_ctx *c) { return boundary(c, R_FLUME); }

af3d_status af3d_force_part(af3d_ctx *c, int sph_id) {
  CHECK_STATE(c);
  if (sph_id < 0 || sph_id > 16) return fail(AF3D_ERR_ARG, "sph_id must be 0..16");
  af3d_status s = ensure_records(c);
  if (s) return s;
  launch_part(c->L(), c->cur, c->d, c->fl_cur, c->nbr, c->cull, c->cells.start, sph_id);
  c->launches++;
  return AF3D_OK;
}

af3d_status af3d_get_accel(af3d_ctx *c) {
  CHECK_STATE(c);
  launch_get_accel(c->L(), c->cur, c->d, c->fl_cur);
  c->launches++;
  return AF3D_OK;
}

af3d_status af3d_finish_verlet(af3d_ctx *c) {
  CHECK_STATE(c);
  launch_finish_verlet(c->L(), c->cur, c->d, c->fl_cur);
  c->launches++;
  c->records_valid = false;
  return AF3D_OK;
}

af3d_status af3d_swap_accel(af3d_ctx *c) {
  CHECK_STATE(c);
  swap_accel_planes(c->cur);
  swap_accel_planes(c->alt);
  return AF3D_OK;
}

af3d_status af3d_forces(af3d_ctx *c) {
  CHECK_STATE(c);
  if (!c->have_grid) return fail(AF3D_ERR_ARG, "no grid");
  AF3D_CUDA(cudaMemsetAsync(&c->d->contacts, 0, sizeof(unsigned long long), c->st));
  enqueue_cell_build(c, false, false);
  c->cells_valid = true;
  // Corrected velocities go to the dead plane set and are dropped: this pass stops at get_accel.
  forces_for(c, true, nullptr, c->alt);
  c->launches += kKernelsPerCellBuild + kKernelsPerForcePass;
  c->records_valid = true;
  int flags = 0;
  af3d_status s = read_status(c, &flags);
  if (s) return s;
  return first_error(flags);
}

af3d_status af3d_step(af3d_ctx *c, long k) {
  CHECK_STATE(c);
  if (k < 0) return fail(AF3D_ERR_ARG, "negative step count");
  if (!c->have_grid) return fail(AF3D_ERR_ARG, "no grid");
  while (k > 0) {
    // The reference re-grids after every step whose counter cc is a multiple of 2000.
    const long to_regrid = (kRegridEvery - c->cc % kRegridEvery) % kRegridEvery;  // steps before it
    const long m = std::min(k, to_regrid + 1);
    af3d_status s = run_steps(c, m);
    if (s) return s;
    for (long i = 0; i < m; i++) c->time = c->time + c->sys[0].dt;
    const bool do_regrid = (c->cc + m - 1) % kRegridEvery == 0;
    c->cc += m;
    k -= m;
    c->cells_valid = true;
    c->records_valid = false;
    if (do_regrid) {
      s = regrid(c);
      if (s) return s;
    }
  }
  int flags = 0;
  af3d_status s = read_status(c, &flags);
  if (s) return s;
  return first_error(flags);
}

af3d_status af3d_prepare_steps(af3d_ctx *c, long k) {
  CHECK_STATE(c);
  if (k < 0) return fail(AF3D_ERR_ARG, "negative step count");
  if (!c->have_grid) return fail(AF3D_ERR_ARG, "no grid");
  // The graphs the next af3d_step(ctx, k) replays up to its first re-grid, captured now (a
  // re-grid may move the cell buffers, so later ones are captured when they come).
  const PtrState p0 = ptr_state(c);
  const long since0 = c->since_sort;
  const bool sorted0 = c->sorted;
  const long to_regrid = (kRegridEvery - c->cc % kRegridEvery) % kRegridEvery;
  const af3d_status s = run_steps(c, std::min(k, to_regrid + 1), false);
  set_ptr_state(c, p0);
  c->since_sort = since0;
  c->sorted = sorted0;
  return s;
}

af3d_status af3d_set_resort_every(af3d_ctx *c, long steps) {
  CHECK_CTX(c);
  if (steps < 2 || steps > 4096 || steps % 2) return fail(AF3D_ERR_ARG, "resort interval: even, 2..4096");
  if (steps != c->resort_every) drop_graphs(c);
  c->resort_every = steps;
  c->since_sort = std::min(c->since_sort, steps);
  return AF3D_OK;
}

af3d_status af3d_set_force_block(af3d_ctx *c, int block) {
  CHECK_CTX(c);
  for (int i = 0; i < kForceShapes; i++)
    if (kForceShapeBlock[i] == block) {
      if (i != c->force_shape) drop_graphs(c);   // graphs hold the force launches' shape
      c->force_shape = i;
      return AF3D_OK;
    }
  return fail(AF3D_ERR_ARG, "force block: 64, 96, 128 or 192 threads");
}

af3d_status af3d_get_force_block(af3d_ctx *c, int *block) {
  CHECK_CTX(c);
  if (!block) return fail(AF3D_ERR_ARG, "null argument");
  *block = kForceShapeBlock[c->force_shape];
  return AF3D_OK;
}

af3d_status af3d_autotune_shapes(af3d_ctx *c, long steps_per_trial, long *resort_every, int *force_block,
                                 double *ms_interval, double *ms_block) {
  CHECK_STATE(c);
  long every = 0;
  af3d_status s = af3d_autotune(c, steps_per_trial, &every, ms_interval);
  if (s) return s;
  // Then each force-kernel shape at that interval: one untimed period (its graph is captured),
  // then whole periods timed, a trial that crossed a re-grid run again.  Results do not depend
  // on the shape, so these are ordinary steps of the run as well.
  cudaEvent_t e0, e1;
  AF3D_CUDA(cudaEventCreate(&e0));
  AF3D_CUDA(cudaEventCreate(&e1));
  struct Events {
    cudaEvent_t a, b;
    ~Events() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } events{e0, e1};
  int best = c->force_shape;
  double best_ms = 0.0;
  const long k = std::max(2 * every, (steps_per_trial + every - 1) / every * every);
  for (int i = 0; i < kForceShapes; i++) {
    s = af3d_set_force_block(c, kForceShapeBlock[i]);
    if (s) return s;
    s = af3d_step(c, every);
    if (s) return s;
    double ms = 0.0;
    for (int attempt = 0; attempt < 2; attempt++) {
      const long cc0 = c->cc;
      AF3D_CUDA(cudaEventRecord(e0, c->st));
      s = af3d_step(c, k);
      if (s) return s;
      AF3D_CUDA(cudaEventRecord(e1, c->st));
      AF3D_CUDA(cudaEventSynchronize(e1));
      float t = 0.0f;
      AF3D_CUDA(cudaEventElapsedTime(&t, e0, e1));
      ms = t / k;
      if (cc0 / kRegridEvery == (c->cc - 1) / kRegridEvery) break;   // no re-grid inside
    }
    if (ms_block) ms_block[i] = ms;
    if (best_ms == 0.0 || ms < best_ms) {
      best_ms = ms;
      best = i;
    }
  }
  s = af3d_set_force_block(c, kForceShapeBlock[best]);
  if (s) return s;
  if (resort_every) *resort_every = every;
  if (force_block) *force_block = kForceShapeBlock[best];
  return AF3D_OK;
}

af3d_status af3d_autotune(af3d_ctx *c, long steps_per_trial, long *resort_every, double *ms_per_step) {
  CHECK_STATE(c);
  if (steps_per_trial < 0) return fail(AF3D_ERR_ARG, "negative trial length");
  if (!c->have_grid) return fail(AF3D_ERR_ARG, "no grid");
  // Every candidate interval: one untimed period (its graph is captured), then whole periods
  // timed; a trial that crossed a re-grid is run again.  Every step taken is a step of the run:
  // the trajectory does not depend on the interval, so tuning costs time only.
  long best = c->resort_every;
  double best_ms = 0.0;
  cudaEvent_t e0, e1;
  AF3D_CUDA(cudaEventCreate(&e0));
  AF3D_CUDA(cudaEventCreate(&e1));
  struct Events {
    cudaEvent_t a, b;
    ~Events() {
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } events{e0, e1};
  int ic = 0;
  for (long cand : kResortChoices) {
    af3d_status s = af3d_set_resort_every(c, cand);
    if (s) return s;
    s = af3d_step(c, cand);
    if (s) return s;
    const long k = std::max(2 * cand, (steps_per_trial + cand - 1) / cand * cand);
    double ms = 0.0;
    for (int attempt = 0; attempt < 2; attempt++) {
      const long cc0 = c->cc;
      AF3D_CUDA(cudaEventRecord(e0, c->st));
      s = af3d_step(c, k);
      if (s) return s;
      AF3D_CUDA(cudaEventRecord(e1, c->st));
      AF3D_CUDA(cudaEventSynchronize(e1));
      float t = 0.0f;
      AF3D_CUDA(cudaEventElapsedTime(&t, e0, e1));
      ms = t / k;
      if (cc0 / kRegridEvery == (c->cc - 1) / kRegridEvery) break;   // no re-grid inside
    }
    if (ms_per_step) ms_per_step[ic] = ms;
    ic++;
    if (best_ms == 0.0 || ms < best_ms) {
      best_ms = ms;
      best = cand;
    }
  }
  af3d_status s = af3d_set_resort_every(c, best);
  if (s) return s;
  if (resort_every) *resort_every = best;
  return AF3D_OK;
}

af3d_status af3d_step_profile(af3d_ctx *c, long k, double *ms) {
  CHECK_STATE(c);
  if (k < 0 || !ms) return fail(AF3D_ERR_ARG, "bad argument");
  if (!c->have_grid) return fail(AF3D_ERR_ARG, "no grid");
  cudaEvent_t ev[AF3D_NPROF + 1];
  for (auto &e : ev) AF3D_CUDA(cudaEventCreate(&e));
  for (long i = 0; i < k; i++) {
    // The steps af3d_step runs, one at a time (the planes are permuted when that is due; a pass
    // looks ahead when the next step keeps the slot order and no re-grid comes between).
    const bool resort = c->since_sort + 1 > c->resort_every;
    const bool warm = !resort && c->look;
    const bool regrid_after = c->cc % kRegridEvery == 0;
    const bool look = i + 1 < k && !regrid_after && !((resort ? 0 : c->since_sort + 1) + 1 > c->resort_every);
    AF3D_CUDA(cudaEventRecord(ev[0], c->st));
    if (!warm) launch_advance_time(c->st, c->d);
    AF3D_CUDA(cudaEventRecord(ev[1], c->st));
    if (!warm) predict_for(c, true, true, true, !resort);
    AF3D_CUDA(cudaEventRecord(ev[2], c->st));
    launch_sort(c->L(), c->d, c->cells, c->id_cur, c->ntags, resort ? nullptr : c->cull, warm);
    AF3D_CUDA(cudaEventRecord(ev[3], c->st));
    if (resort) {
      launch_permute_records(c->L(), c->cur, c->alt, c->cells.perm, c->id_cur, c->id_alt, c->fl_cur,
                             c->fl_alt, c->nbr, c->cull, false);
      std::swap(c->cur, c->alt);
      std::swap(c->id_cur, c->id_alt);
      std::swap(c->fl_cur, c->fl_alt);
    }
    AF3D_CUDA(cudaEventRecord(ev[4], c->st));
    if (resort) {
      forces_for(c, false, nullptr, c->alt, false, look);
      swap_velocity_planes(c->cur, c->alt);
    } else {
      forces_for(c, false, c->cells.perm, c->cur, warm, look);
    }
    if (look) {
      std::swap(c->nbr, c->nbr_next);
      std::swap(c->cull, c->cull_next);
    }
    c->look = look;
    swap_accel_planes(c->cur);
    swap_accel_planes(c->alt);
    AF3D_CUDA(cudaEventRecord(ev[5], c->st));
    c->sorted = resort;
    c->since_sort = resort ? 0 : c->since_sort + 1;
    c->launches += kernels_of(1, resort, warm);
    c->time = c->time + c->sys[0].dt;
    const bool do_regrid = c->cc % kRegridEvery == 0;
    c->cc++;
    if (do_regrid) {
      af3d_status s = regrid(c);
      if (s) return s;
    }
    AF3D_CUDA(cudaEventRecord(ev[6], c->st));
    AF3D_CUDA(cudaEventSynchronize(ev[6]));
    for (int p = 0; p < AF3D_NPROF; p++) {
      float t = 0.f;
      AF3D_CUDA(cudaEventElapsedTime(&t, ev[p], ev[p + 1]));
      ms[p] += t;
    }
    c->cells_valid = !do_regrid;
  }
  for (auto &e : ev) cudaEventDestroy(e);
  c->records_valid = false;
  int flags = 0;
  af3d_status s = read_status(c, &flags);
  if (s) return s;
  return first_error(flags);
}

af3d_status af3d_kernel_launches(af3d_ctx *c, long *count) {
  CHECK_CTX(c);
  if (!count) return fail(AF3D_ERR_ARG, "null argument");
  *count = c->launches;
  return AF3D_OK;
}

af3d_status af3d_check_fp64_bits(const double *x, long n, int *bad) {
  if (n < 0 || (n > 0 && (!x || !bad))) return fail(AF3D_ERR_ARG, "bad argument");
  AF3D_CUDA(check_fp64_bits(x, n, bad));
  return AF3D_OK;
}

af3d_status af3d_fp64_peak(double *tflops) {
  if (!tflops) return fail(AF3D_ERR_ARG, "null argument");
  int dev = 0, sms = 0;
  AF3D_CUDA(cudaGetDevice(&dev));
  AF3D_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double best = 0.0;
  for (int rep = 0; rep < 3; rep++) {
    double t = 0.0;
    AF3D_CUDA(measure_dfma(sms, &t));
    best = std::max(best, t);
  }
  *tflops = best;
  return AF3D_OK;
}

af3d_status af3d_get_status(af3d_ctx *c, int *flags) {
  CHECK_CTX(c);
  if (!flags) return fail(AF3D_ERR_ARG, "null argument");
  return read_status(c, flags);
}

af3d_status af3d_get_forces(af3d_ctx *c, af3d_vec3 *force, af3d_vec3 *torque) {
  CHECK_STATE(c);
  return gather_by_id(c, FX, force, torque);
}

af3d_status af3d_get_accels(af3d_ctx *c, af3d_vec3 *acc_f, af3d_vec3 *anga_f) {
  CHECK_STATE(c);
  return gather_by_id(c, AFX, acc_f, anga_f);
}

af3d_status af3d_get_cells(af3d_ctx *c, long *cell_of_id, long *sorted_ids, long *nbinned) {
  CHECK_STATE(c);
  if (!c->cells_valid) return fail(AF3D_ERR_ARG, "no cell build since the last grid change");
  if (!c->sorted) return fail(AF3D_ERR_ARG, "af3d_step left the slots out of cell order: call af3d_cell_build");
  if (c->n == 0) {
    if (nbinned) *nbinned = 0;
    return AF3D_OK;
  }
  if (!c->d_tmp) AF3D_CUDA(cudaMalloc(&c->d_tmp, sizeof(long long) * c->n));
  long long total = 0;
  AF3D_CUDA(cudaMemcpyAsync(&total, &c->d->ncell_total, sizeof(total), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  int nb = 0;
  AF3D_CUDA(cudaMemcpy(&nb, c->cells.start + total, sizeof(int), cudaMemcpyDeviceToHost));
  if (nbinned) *nbinned = nb;
  if (cell_of_id) {
    // keys belong to the layout before the last permutation, whose ids are now in id_alt
    launch_cells_by_id(c->L(), c->cells.key, c->id_alt, c->d, c->d_tmp);
    AF3D_CUDA(cudaMemcpyAsync(cell_of_id, c->d_tmp, sizeof(long long) * c->n, cudaMemcpyDeviceToHost, c->st));
  }
  if (sorted_ids && nb > 0)
    AF3D_CUDA(cudaMemcpyAsync(sorted_ids, c->id_cur, sizeof(long long) * nb, cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  return AF3D_OK;
}

af3d_status af3d_contact_pairs(af3d_ctx *c, long *out, long cap, long *count, int active) {
  CHECK_STATE(c);
  af3d_status s = ensure_records(c);
  if (s) return s;
  // the staging buffer is freed on every exit path, the early error returns included
  struct Staging {
    long long *p = nullptr;
    ~Staging() { if (p) cudaFree(p); }
  } staging;
  if (cap > 0) AF3D_CUDA(cudaMalloc(&staging.p, sizeof(long long) * 3 * cap));
  long long *d_out = staging.p;
  AF3D_CUDA(cudaMemsetAsync(c->d_count, 0, sizeof(unsigned long long), c->st));
  launch_contact_pairs(c->L(), c->cur, c->d, c->fl_cur, c->nbr, c->cull, c->cells.start, c->id_cur, d_out,
                       c->d_count, cap, active);
  unsigned long long cnt = 0;
  AF3D_CUDA(cudaMemcpyAsync(&cnt, c->d_count, sizeof(cnt), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  if (count) *count = (long)cnt;
  if (cap > 0 && out)
    AF3D_CUDA(cudaMemcpy(out, d_out, sizeof(long long) * 3 * std::min<long>(cap, (long)cnt),
                         cudaMemcpyDeviceToHost));
  return AF3D_OK;
}

af3d_status af3d_contact_count(af3d_ctx *c, long *count) {
  CHECK_CTX(c);
  if (!count) return fail(AF3D_ERR_ARG, "null argument");
  unsigned long long v = 0, zero = 0;
  AF3D_CUDA(cudaMemcpyAsync(&v, &c->d->contacts, sizeof(v), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaMemcpyAsync(&c->d->contacts, &zero, sizeof(zero), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  *count = (long)v;
  return AF3D_OK;
}

af3d_status af3d_list_overflows(af3d_ctx *c, long *count) {
  CHECK_CTX(c);
  if (!count) return fail(AF3D_ERR_ARG, "null argument");
  unsigned long long v = 0, zero = 0;
  AF3D_CUDA(cudaMemcpyAsync(&v, &c->d->overflows, sizeof(v), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaMemcpyAsync(&c->d->overflows, &zero, sizeof(zero), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  *count = (long)v;
  return AF3D_OK;
}

}  // extern "C"

// ---- allocation-free contact-pair readout ----------------------------------------------------
//
// af3d_contact_pairs stages the pairs in a device buffer it allocates and frees on every call.
// Some callers cannot allow that: a host framework that reserved the GPU's memory for its own
// caching pool at start-up would see the allocation fail mid-run, and cudaMalloc/cudaFree
// around a diagnostic synchronise the whole device, stalling every other stream of a running
// simulation.  af3d_contact_pairs_noalloc runs the same contact-pair kernel on a fixed staging
// array that is part of this library's device image, so a call allocates no device memory.
//
// Set-up: the first call on a device, made with that device current, looks up the array's
// device address once (cudaGetSymbolAddress; this also loads the library's device image on that
// device if nothing else has).  Make that first call before any stream capture begins.
// Sharing: every context on a device uses the same array, so calls that overlap in time (from
// two host threads, or on two streams) race on it; callers serialise them per device.
namespace {

constexpr long kNoAllocMaxPairs = 262144;   // at most 262,144 (ll, mm, sph_id) triples: 6 MiB
constexpr size_t kNoAllocHead = 256;        // the pair counter, padded to the array alignment
constexpr int kNoAllocMaxDevices = 64;

// [0, 8): pair counter, zeroed on the stream before each launch; [256, ...): the triples.
static __device__ __align__(256) unsigned char
    g_noalloc_scratch[kNoAllocHead + sizeof(long long) * 3 * kNoAllocMaxPairs];

std::mutex g_noalloc_mutex;
unsigned char *g_noalloc_addr[kNoAllocMaxDevices] = {};

af3d_status noalloc_scratch(int device, unsigned char **addr) {
  if (device < 0 || device >= kNoAllocMaxDevices)
    return fail(AF3D_ERR_ARG, "device index beyond the " + std::to_string(kNoAllocMaxDevices) +
                                  " devices the staging table covers");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(AF3D_ERR_CUDA, std::string("cudaGetSymbolAddress(staging array): ") + cudaGetErrorString(e));
    g_noalloc_addr[device] = static_cast<unsigned char *>(p);
  }
  *addr = g_noalloc_addr[device];
  return AF3D_OK;
}

}  // namespace

extern "C" af3d_status af3d_contact_pairs_noalloc(af3d_ctx *c, long *out, long cap, long *count, int active) {
  CHECK_STATE(c);
  if (cap < 0 || cap > kNoAllocMaxPairs)
    return fail(AF3D_ERR_ARG, "cap " + std::to_string(cap) + " is outside [0, " +
                                  std::to_string(kNoAllocMaxPairs) + "], the staging array's size in pairs");
  if (cap > 0 && !out) return fail(AF3D_ERR_ARG, "null output array");
  int device = -1;
  AF3D_CUDA(cudaGetDevice(&device));
  if (device != c->device) return fail(AF3D_ERR_ARG, "the context's device must be the current device");
  unsigned char *scratch = nullptr;
  af3d_status s = noalloc_scratch(device, &scratch);
  if (s) return s;
  s = ensure_records(c);
  if (s) return s;
  unsigned long long *d_count = reinterpret_cast<unsigned long long *>(scratch);
  long long *d_out = reinterpret_cast<long long *>(scratch + kNoAllocHead);
  AF3D_CUDA(cudaMemsetAsync(d_count, 0, sizeof(unsigned long long), c->st));   // counter starts at 0
  launch_contact_pairs(c->L(), c->cur, c->d, c->fl_cur, c->nbr, c->cull, c->cells.start, c->id_cur, d_out,
                       d_count, cap, active);
  unsigned long long cnt = 0;
  AF3D_CUDA(cudaMemcpyAsync(&cnt, d_count, sizeof(cnt), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  const long kept = std::min<long>(cap, (long)cnt);
  if (kept > 0) {
    AF3D_CUDA(cudaMemcpyAsync(out, d_out, sizeof(long long) * 3 * kept, cudaMemcpyDeviceToHost, c->st));
    AF3D_CUDA(cudaStreamSynchronize(c->st));
  }
  AF3D_CUDA(cudaGetLastError());
  if (count) *count = (long)cnt;
  return AF3D_OK;
}

// ---- adjoint of the exact step ----------------------------------------------------------------
namespace {

// Device buffers of the adjoint run, freed on every exit path.
struct AdjBuffers {
  std::vector<void *> owned;
  ~AdjBuffers() {
    for (void *p : owned) cudaFree(p);
  }
  cudaError_t planes(int k, long n, Planes &P) {
    double *base = nullptr;
    const cudaError_t e = cudaMalloc((void **)&base, sizeof(double) * (size_t)k * (size_t)n);
    if (e != cudaSuccess) return e;
    owned.push_back(base);
    for (int i = 0; i < NPLANES; i++) P.p[i] = i < k ? base + (size_t)i * n : nullptr;
    return cudaSuccess;
  }
};

af3d_status set_device_time(af3d_ctx *c, double t) {
  AF3D_CUDA(cudaMemcpyAsync(&c->d->time, &t, sizeof(double), cudaMemcpyHostToDevice, c->st));
  return AF3D_OK;
}

// The start-up force pass without moving the slots: keys and records at the current positions,
// the sort, and every force of the phase into F, T and a_f.
void enqueue_startup_pass(af3d_ctx *c) {
  predict_for(c, false, true, false, true);
  launch_sort(c->L(), c->d, c->cells, c->id_cur, c->ntags, c->cull);
  forces_for(c, true, c->cells.perm, c->alt);   // corrected velocities go to the dead set
}

// This step's cell structure at the recomputed predicted state (records, keys, sort).
void enqueue_step_cells(af3d_ctx *c) {
  launch_advance_time(c->st, c->d);
  predict_for(c, true, true, true, true);
  launch_sort(c->L(), c->d, c->cells, c->id_cur, c->ntags, c->cull);
}

// The plane set with its torque planes replaced by planes 24..26 of a tape slot.
Planes with_tape_torque(Planes P, const Planes &tape) {
  for (int k = 0; k < 3; k++) P.p[TX + k] = tape.p[kAdjPlanes + k];
  return P;
}

}  // namespace

extern "C" af3d_status af3d_adjoint(af3d_ctx *c, long steps, long ckpt_every, double *J, double *param_grad,
                                    af3d_vec3 *dr0, double *dR0, af3d_vec3 *dv0, af3d_vec3 *dw0) {
  CHECK_STATE(c);
  if (steps < 0 || ckpt_every <= 0 || !J) return fail(AF3D_ERR_ARG, "bad argument");
  if (!c->have_grid) return fail(AF3D_ERR_ARG, "no grid");
  const long n = c->n;
  const int nf = c->nflumes;
  const bool want_grad = param_grad || dr0 || dR0 || dv0 || dw0;
  const int mode = c->fp_mode;
  c->fp_mode = AF3D_FP_EXACT;   // the adjoint differentiates the exact step
  struct ModeBack {
    af3d_ctx *c;
    int m;
    ~ModeBack() { c->fp_mode = m; }
  } mode_back{c, mode};
  drop_graphs(c);
  AdjBuffers buf;
  Planes state0{}, fin{}, adjA{}, adjB{}, acc{}, rb{}, rnext{};
  cudaError_t e = buf.planes(kAdjPlanes + 12, n, state0);   // with the sphere centres
  if (e == cudaSuccess) e = buf.planes(kAdjPlanes + 12, n, fin);
  if (want_grad && e == cudaSuccess) e = buf.planes(kAdjPlanes, n, adjA);
  if (want_grad && e == cudaSuccess) e = buf.planes(kAdjPlanes, n, adjB);
  if (want_grad && e == cudaSuccess) e = buf.planes(kAccPlanes, n, acc);
  if (want_grad && e == cudaSuccess) e = buf.planes(kRbPlanes, n, rb);
  if (want_grad && e == cudaSuccess) e = buf.planes(9, n, rnext);
  // The tape: per step its starting state and torque sums (27 planes), its clump records, item
  // lists and list counts, in one block.  It holds C = ckpt_every steps when they fit in the
  // free device memory (with a reserve), else the largest C, halving, that does: the results do
  // not depend on C.  Checkpoints open every segment but the last, which the forward run tapes
  // itself.
  const size_t m = (size_t)std::max<long>(n, 1);
  const size_t slot = (sizeof(double) * (kAdjPlanes + 3) * m + sizeof(NbrRec) * m +
                       (sizeof(unsigned) * kListCap + sizeof(int)) * m + 255) & ~(size_t)255;
  const size_t ckpt_bytes = sizeof(double) * kAdjPlanes * m;
  long C = std::min(ckpt_every, std::max<long>(steps, 1));
  if (want_grad && e == cudaSuccess) {
    size_t free_b = 0, total_b = 0;
    e = cudaMemGetInfo(&free_b, &total_b);
    const size_t reserve = (size_t)2 << 30;
    const size_t avail = free_b > reserve ? free_b - reserve : 0;
    auto need = [&](long cseg) {
      const long nck_c = steps > 0 ? (steps - 1) / cseg : 0;
      return slot * (size_t)cseg + ckpt_bytes * (size_t)nck_c;
    };
    while (C > 1 && need(C) > avail) C = (C + 1) / 2;
  }
  const long nck = steps > 0 ? (steps - 1) / C : 0;
  std::vector<Planes> ckpt(want_grad ? nck : 0), tape(want_grad ? C : 0);
  std::vector<ContactLists> tape_lists(tape.size());
  std::vector<NbrRec *> tape_rec(tape.size());
  for (size_t k = 0; k < ckpt.size() && e == cudaSuccess; k++) e = buf.planes(kAdjPlanes, n, ckpt[k]);
  if (!tape.empty() && e == cudaSuccess) {
    char *base = nullptr;
    e = cudaMalloc((void **)&base, slot * tape.size());
    if (e == cudaSuccess) {
      buf.owned.push_back(base);
      for (size_t k = 0; k < tape.size(); k++) {
        double *pl = reinterpret_cast<double *>(base + slot * k);
        for (int i = 0; i < NPLANES; i++) tape[k].p[i] = i < kAdjPlanes + 3 ? pl + (size_t)i * m : nullptr;
        tape_rec[k] = reinterpret_cast<NbrRec *>(pl + (size_t)(kAdjPlanes + 3) * m);
        tape_lists[k].items = reinterpret_cast<unsigned *>(tape_rec[k] + m);
        tape_lists[k].cnt = reinterpret_cast<int *>(tape_lists[k].items + (size_t)kListCap * m);
        tape_lists[k].ovf = nullptr;
      }
    }
  }
  // per flume f: dsc[3 f .. 3 f + 2] the objective sums, pgr[6 f .. 6 f + 5] the parameter
  // adjoints; then per step: its list overflow flag (int), its start and end times (a pair)
  const size_t nsc = (size_t)9 * nf;
  double *dsc = nullptr;
  if (e == cudaSuccess) e = cudaMalloc((void **)&dsc, sizeof(double) * (nsc + 3 * (size_t)(steps + 1)));
  if (e == cudaSuccess) buf.owned.push_back(dsc);
  if (e != cudaSuccess) return fail(AF3D_ERR_NOMEM, std::string("adjoint buffers: ") + cudaGetErrorString(e));
  double *pgr = dsc + 3 * nf;
  double *t_pair = dsc + nsc;   // [steps + 1][2]: {time, time_prev} during step k
  int *ovf = reinterpret_cast<int *>(t_pair + 2 * (size_t)(steps + 1));
  AF3D_CUDA(cudaMemsetAsync(dsc, 0, sizeof(double) * (nsc + 3 * (size_t)(steps + 1)), c->st));

  // The context's own record buffers, item lists and torque planes, put back on every exit.
  struct OwnPointers {
    af3d_ctx *c;
    NbrRec *nbr, *nbr_next;
    ContactLists lists;
    double *tq[3];
    void restore() {
      c->nbr = nbr;
      c->nbr_next = nbr_next;
      c->lists = lists;
      for (int q = 0; q < 3; q++) c->cur.p[TX + q] = tq[q];
    }
    ~OwnPointers() { restore(); }
  } own{c, c->nbr, c->nbr_next, c->lists, {c->cur.p[TX], c->cur.p[TX + 1], c->cur.p[TX + 2]}};

  // Forward: the start-up force pass (a_i of the first step), then `steps` steps keeping the
  // slot order, the state saved every C steps.
  const double t_init = c->time, dt = c->sys[0].dt;
  launch_state_copy(c->L(), c->cur, state0, true, true);
  enqueue_startup_pass(c);
  c->look = false;   // records of a previous run's look-ahead are stale now
  swap_accel_planes(c->cur);
  swap_accel_planes(c->alt);
  // The last segment's steps record their tape slots here (the reverse starts with them).
  const long seg_last = steps > 0 ? (steps - 1) / C : 0, k_last = seg_last * C;
  // Step k of a segment [k0, k1) into its tape slot: its starting state, its clump records
  // (written by the previous pass's look-ahead, or by this step's predictor), item lists, list
  // counts and torque sums.  A kept-order step neither swaps nor reallocates the plane sets, and
  // the record buffers only swap, so pointing them at the tape is enough.
  auto taped_step = [&](long k, long k0, long k1) {
    launch_state_copy(c->L(), c->cur, tape[k - k0], true);
    if (!c->look) c->nbr = tape_rec[k - k0];
    if (k + 1 < k1) c->nbr_next = tape_rec[k + 1 - k0];
    c->lists = tape_lists[k - k0];
    c->lists.ovf = ovf + k;
    c->cur = with_tape_torque(c->cur, tape[k - k0]);
    enqueue_fused_step(c, false, true, k + 1 < k1);
    for (int q = 0; q < 3; q++) c->cur.p[TX + q] = own.tq[q];
    c->lists = own.lists;
  };
  std::vector<double> t_start(steps + 1);
  double t = t_init;
  for (long k = 0; k < steps; k++) {
    t_start[k] = t;
    if (want_grad && k >= k_last) {
      taped_step(k, k_last, steps);
    } else {
      if (want_grad && k % C == 0) launch_state_copy(c->L(), c->cur, ckpt[k / C], true);
      if (want_grad && k + 1 == k_last) c->nbr_next = tape_rec[0];   // the taped segment's first records
      enqueue_fused_step(c, false, false, k + 1 < steps);   // the last pass does not look ahead
    }
    t = t + dt;
  }
  own.restore();
  t_start[steps] = t;
  c->time = t;
  launch_state_copy(c->L(), c->cur, fin, true, true);
  launch_adj_objective(c->L(), c->cur, c->d, c->fl_cur, dsc, c->obj_length);
  std::vector<double> sums((size_t)3 * nf);
  std::vector<int> ovf_h(steps + 1, 0);
  AF3D_CUDA(cudaMemcpyAsync(sums.data(), dsc, sizeof(double) * 3 * nf, cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaMemcpyAsync(ovf_h.data(), ovf, sizeof(int) * (steps + 1), cudaMemcpyDeviceToHost, c->st));
  int flags = 0;
  af3d_status s = read_status(c, &flags);
  if (s) return s;
  s = first_error(flags);
  if (s) return s;
  for (int f = 0; f < nf; f++) {
    const double S = sums[3 * f], M = sums[3 * f + 1];
    if (!(M > 0.0)) {
      J[f] = 0.0;
    } else if (c->obj_length > 0.0) {
      uint64_t key;   // x_max as the device's order-preserving integer
      std::memcpy(&key, &sums[3 * f + 2], sizeof key);
      const uint64_t u = (key >> 63) ? (key & 0x7fffffffffffffffull) : ~key;
      double xmax;
      std::memcpy(&xmax, &u, sizeof xmax);
      J[f] = xmax + c->obj_length * std::log(S / M);
    } else {
      J[f] = S / M;
    }
  }

  if (want_grad && n > 0) {
    // every step's times on the device (set by device-side copies, the host runs ahead): step k
    // runs at time t_start[k + 1] after its clock advance, with time_prev t_start[k]
    std::vector<double> tp(2 * (size_t)(steps + 1), 0.0);
    for (long k = 0; k < steps; k++) {
      tp[2 * k] = t_start[k + 1];
      tp[2 * k + 1] = t_start[k];
    }
    static_assert(offsetof(DevScalars, time_prev) == offsetof(DevScalars, time) + sizeof(double), "time pair");
    AF3D_CUDA(cudaMemcpyAsync(t_pair, tp.data(), sizeof(double) * tp.size(), cudaMemcpyHostToDevice, c->st));
    launch_adj_seed(c->L(), c->cur, adjA, c->d, c->fl_cur, dsc, c->obj_length);
    Planes rnext_src = fin;   // R1 of each segment's last step: the next segment's starting R
    for (long seg = (steps - 1) / C; steps > 0 && seg >= 0; seg--) {
      const long k0 = seg * C, k1 = std::min(steps, k0 + C);
      // recompute the segment into the tape (the last one was taped by the forward run)
      if (seg != seg_last) {
        for (int q = 0; q < 9; q++)   // tape slot 0 still holds segment seg + 1's starting state
          AF3D_CUDA(cudaMemcpyAsync(rnext.p[q], tape[0].p[R00 + q], sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                    c->st));
        for (int q = 0; q < 9; q++) rnext_src.p[R00 + q] = rnext.p[q];
        launch_state_copy(c->L(), c->cur, ckpt[seg], false);
        c->look = false;   // the restored state has not been predicted
        AF3D_CUDA(cudaMemcpyAsync(&c->d->time, t_pair + 2 * k0 + 1, sizeof(double), cudaMemcpyDeviceToDevice,
                                  c->st));
        for (long k = k0; k < k1; k++) taped_step(k, k0, k1);
        own.restore();
        AF3D_CUDA(cudaMemcpyAsync(ovf_h.data() + k0, ovf + k0, sizeof(int) * (k1 - k0), cudaMemcpyDeviceToHost,
                                  c->st));
        AF3D_CUDA(cudaStreamSynchronize(c->st));
      }
      // then each step backwards from its tape slot: records, lists, torque sums, and R1 (the
      // next step's starting R).  A step whose lists overflowed rebuilds its cell structure for
      // the per-clump walk of the overflowed clumps.
      for (long k = k1 - 1; k >= k0; k--) {
        AF3D_CUDA(cudaMemcpyAsync(&c->d->time, t_pair + 2 * k, 2 * sizeof(double), cudaMemcpyDeviceToDevice, c->st));
        Planes Pk = with_tape_torque(c->cur, tape[k - k0]);
        const Planes &r1 = k + 1 < k1 ? tape[k + 1 - k0] : rnext_src;
        for (int q = 0; q < 9; q++) Pk.p[R00 + q] = r1.p[R00 + q];
        const NbrRec *rec = tape_rec[k - k0];
        if (ovf_h[k]) {
          launch_state_copy(c->L(), c->cur, tape[k - k0], false);
          AF3D_CUDA(cudaMemcpyAsync(&c->d->time, t_pair + 2 * k + 1, sizeof(double), cudaMemcpyDeviceToDevice,
                                    c->st));
          enqueue_step_cells(c);   // the same records again, and the cells
          rec = c->nbr;
        }
        AF3D_CUDA(cudaMemsetAsync(acc.p[0], 0, sizeof(double) * kAccPlanes * n, c->st));   // one block
        launch_adj_forces_lists(c->L(), Pk, adjA, adjB, acc, rb, c->d, c->fl_cur, rec, c->cull, c->cells.start,
                                c->cells.perm, tape_lists[k - k0], pgr);
        launch_adj_predict(c->L(), Pk, tape[k - k0], adjA, adjB, acc, rb, c->d, c->fl_cur);
        std::swap(adjA, adjB);
      }
    }
    // the start-up pass backwards
    launch_state_copy(c->L(), c->cur, state0, false, true);
    s = set_device_time(c, t_init);
    if (s) return s;
    enqueue_startup_pass(c);
    AF3D_CUDA(cudaMemsetAsync(acc.p[0], 0, sizeof(double) * kAccPlanes * n, c->st));
    launch_adj_forces(c->L(), c->cur, adjA, adjB, acc, rb, c->d, c->fl_cur, c->nbr, c->cull, c->cells.start,
                      c->cells.perm, c->cells.csort, pgr, true);
    launch_adj_startup(c->L(), c->cur, adjA, adjB, acc, rb);
    // gradients by clump id
    std::vector<double> h((size_t)kAdjPlanes * n);
    std::vector<long long> ids(n);
    for (int p = 0; p < kAdjPlanes; p++)
      AF3D_CUDA(cudaMemcpyAsync(h.data() + (size_t)p * n, adjB.p[p], sizeof(double) * n, cudaMemcpyDeviceToHost,
                                c->st));
    AF3D_CUDA(cudaMemcpyAsync(ids.data(), c->id_cur, sizeof(long long) * n, cudaMemcpyDeviceToHost, c->st));
    if (param_grad)
      AF3D_CUDA(cudaMemcpyAsync(param_grad, pgr, sizeof(double) * 6 * nf, cudaMemcpyDeviceToHost, c->st));
    AF3D_CUDA(cudaStreamSynchronize(c->st));
    for (long sl = 0; sl < n; sl++) {
      const long long i = ids[sl];
      auto at = [&](int p) { return h[(size_t)p * n + sl]; };
      if (dr0) dr0[i] = {at(0), at(1), at(2)};
      if (dv0) dv0[i] = {at(3), at(4), at(5)};
      if (dw0) dw0[i] = {at(6), at(7), at(8)};
      if (dR0)
        for (int k = 0; k < 9; k++) dR0[9 * i + k] = at(9 + k);
    }
  }
  // leave the context at the final state of the forward run
  launch_state_copy(c->L(), c->cur, fin, false, true);
  s = set_device_time(c, t);
  if (s) return s;
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  c->sorted = false;
  c->records_valid = false;
  c->cells_valid = false;
  c->look = false;
  c->since_sort = c->resort_every;
  c->cc += steps;
  flags = 0;
  s = read_status(c, &flags);
  if (s) return s;
  return first_error(flags);
}
