// af3d_capi.cu -- host side of the C ABI declared in include/af3d.h.
//
// The context owns every device buffer; the reference's caller-owned arrays become planes of a
// structure-of-arrays state kept in cell-sorted order.  The per-routine entry points enqueue one
// kernel (or the cell build) each on the context stream and return; af3d_step() enqueues whole
// fused steps and replays them from CUDA graphs.  Device-side checks raise bits in a status word
// that af3d_step() and af3d_get_status() read back; nothing calls exit().
#include <algorithm>
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
constexpr long kKernelsPerCellBuild = 7;   // predict/keys, 3 scan, scatter, rank, permute
constexpr long kKernelsPerStep = kKernelsPerCellBuild + 2;   // + time advance, fused forces
constexpr long kKernelsPerRegrid = 3;

struct StepGraph {
  Planes cur, alt;
  long long *id_cur = nullptr;
  cudaGraphExec_t exec = nullptr;
};

}  // namespace

struct af3d_ctx {
  int device = 0;
  long n = 0;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  af3d_system_par sys{};     // host mirror (time advanced in step with the device)
  af3d_funnel fun{};
  af3d_cell_par grid{};      // host mirror, refreshed from the device after a device re-grid
  bool have_grid = false;
  long ntags = 9;
  int phase = AF3D_PHASE_AVALANCHE;
  int variant = AF3D_FRICTION_HST;
  long cc = 0;               // steps done in the current phase
  bool imported = false;

  double *plane_mem[2] = {nullptr, nullptr};
  Planes cur{}, alt{};
  long long *id_cur = nullptr, *id_alt = nullptr;
  NbrRec *nbr = nullptr;
  CullRec *cull = nullptr;
  Cells cells{};
  DevScalars *d = nullptr;
  bool records_valid = false;   // records reflect the current planes
  bool cells_valid = false;     // start[] describes the current layout

  af3d_particle *d_aos = nullptr;
  double *d_acc = nullptr, *d_anga = nullptr;
  long long *d_tmp = nullptr;
  unsigned long long *d_count = nullptr;

  StepGraph graphs[2];
  int graph_next = 0;
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

void drop_graphs(af3d_ctx *c) {
  for (auto &g : c->graphs) {
    if (g.exec) cudaGraphExecDestroy(g.exec);
    g = StepGraph{};
  }
}

af3d_status push_scalars(af3d_ctx *c) {
  // Host-side system/grid edits go to the device on the context stream (ordered with kernels).
  AF3D_CUDA(cudaMemcpyAsync(&c->d->sys, &c->sys, sizeof(af3d_system_par), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaMemcpyAsync(&c->d->fun, &c->fun, sizeof(af3d_funnel), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaMemcpyAsync(&c->d->phase, &c->phase, sizeof(int), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaMemcpyAsync(&c->d->variant, &c->variant, sizeof(int), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  return AF3D_OK;
}

af3d_status ensure_buckets(af3d_ctx *c, long ncell3) {
  const long need = ncell3 + c->n + 1;
  if (need <= c->cells.cap && c->cells.count) return AF3D_OK;
  const long cap = std::max<long>(need + need / 2, 1024);
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  cudaFree(c->cells.count);
  cudaFree(c->cells.start);
  cudaFree(c->cells.block_sums);
  c->cells.count = c->cells.start = c->cells.block_sums = nullptr;
  AF3D_CUDA(cudaMalloc(&c->cells.count, sizeof(int) * cap));
  AF3D_CUDA(cudaMalloc(&c->cells.start, sizeof(int) * (cap + 1)));
  AF3D_CUDA(cudaMalloc(&c->cells.block_sums, sizeof(int) * (scan_tiles(cap) + 1)));
  AF3D_CUDA(cudaMemsetAsync(c->cells.count, 0, sizeof(int) * cap, c->st));
  c->cells.cap = cap;
  c->cells_valid = false;
  drop_graphs(c);
  return AF3D_OK;
}

af3d_status set_grid_device(af3d_ctx *c, const af3d_cell_par &g) {
  af3d_status s = ensure_buckets(c, g.ncell3);
  if (s) return s;
  c->grid = g;
  c->have_grid = true;
  AF3D_CUDA(cudaMemcpyAsync(&c->d->grid, &c->grid, sizeof(af3d_cell_par), cudaMemcpyHostToDevice, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  c->cells_valid = false;
  return AF3D_OK;
}

// Device re-grid, then adopt the result on the host (grow the bucket buffers if needed).
af3d_status regrid(af3d_ctx *c) {
  if (c->n == 0) return AF3D_OK;   // no clump to bound (cell_dim reads pp[0]): keep the grid
  launch_regrid(c->L(), c->cur, c->d, c->cells.cap);
  c->launches += kKernelsPerRegrid;
  long long pending = 0;
  AF3D_CUDA(cudaMemcpyAsync(&pending, &c->d->pending_ncell3, sizeof(long long), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  if (pending < 0) return fail(AF3D_ERR_GRID_ESCAPE, "re-grid produced an empty grid");
  if (pending > 0) {
    af3d_cell_par g;
    AF3D_CUDA(cudaMemcpy(&g, &c->d->pending, sizeof(g), cudaMemcpyDeviceToHost));
    return set_grid_device(c, g);
  }
  AF3D_CUDA(cudaMemcpy(&c->grid, &c->d->grid, sizeof(af3d_cell_par), cudaMemcpyDeviceToHost));
  c->have_grid = true;
  return AF3D_OK;
}

// clear_cell + clear_ocup + cell_locate: keys (optionally fused with the predictor), counting
// sort, permutation of every plane into the new order, neighbour records.
void enqueue_cell_build(af3d_ctx *c, bool predict, bool t_prev, bool ft = true) {
  launch_predict(c->L(), c->cur, c->d, predict, true, t_prev, c->cells, c->id_cur);
  launch_sort(c->L(), c->d, c->cells, c->id_cur, c->ntags);
  launch_permute_records(c->L(), c->cur, c->alt, c->cells.perm, c->id_cur, c->id_alt, c->nbr, c->cull, ft);
  std::swap(c->cur, c->alt);
  std::swap(c->id_cur, c->id_alt);
}

// One fused step: time += dt, init_Verlet + cell build, every force of the phase, get_accel,
// finish_Verlet, and the acceleration swap.
void enqueue_fused_step(af3d_ctx *c) {
  launch_advance_time(c->st, c->d);
  enqueue_cell_build(c, true, true, false);   // F, T are not read by the fused force kernel
  launch_fused_forces(c->L(), c->cur, c->alt, c->d, c->nbr, c->cull, c->cells.start, false);
  swap_velocity_planes(c->cur, c->alt);
  swap_accel_planes(c->cur);
  swap_accel_planes(c->alt);
}

af3d_status run_steps(af3d_ctx *c, long m) {
  // Pairs of steps return the plane pointers to where they started, so a captured two-step
  // graph can be replayed; an odd step is enqueued directly.
  while (m >= 2) {
    StepGraph *g = nullptr;
    for (auto &cand : c->graphs)
      if (cand.exec && cand.id_cur == c->id_cur && same_planes(cand.cur, c->cur) &&
          same_planes(cand.alt, c->alt))
        g = &cand;
    if (!g) {
      g = &c->graphs[c->graph_next];
      c->graph_next ^= 1;
      if (g->exec) cudaGraphExecDestroy(g->exec);
      *g = StepGraph{};
      g->cur = c->cur;
      g->alt = c->alt;
      g->id_cur = c->id_cur;
      cudaGraph_t graph;
      AF3D_CUDA(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
      enqueue_fused_step(c);
      enqueue_fused_step(c);
      AF3D_CUDA(cudaStreamEndCapture(c->st, &graph));
      cudaError_t e = cudaGraphInstantiate(&g->exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) {
        g->exec = nullptr;
        return fail(AF3D_ERR_CUDA, std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e));
      }
    }
    AF3D_CUDA(cudaGraphLaunch(g->exec, c->st));
    c->launches += 2 * kKernelsPerStep;
    m -= 2;
  }
  if (m == 1) {
    enqueue_fused_step(c);
    c->launches += kKernelsPerStep;
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
  if (!c->records_valid) {
    launch_build_records(c->L(), c->cur, c->nbr, c->cull);
    c->records_valid = true;
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

}  // namespace

extern "C" {

const char *af3d_last_error(void) { return g_last_error.c_str(); }
int af3d_abi_version(void) { return AF3D_ABI_VERSION; }

af3d_status af3d_create(const af3d_system_par *sys, const af3d_funnel *fun, long ntags, int phase,
                        af3d_ctx **out) {
  if (!sys || !fun || !out) return fail(AF3D_ERR_ARG, "null argument");
  if (sys->npart < 0 || sys->npart > (1L << 28)) return fail(AF3D_ERR_ARG, "npart out of range (0..2^28)");
  *out = nullptr;
  af3d_ctx *c = new af3d_ctx();
  c->n = sys->npart;
  c->sys = *sys;
  c->fun = *fun;
  c->ntags = ntags;
  c->phase = phase;
  cudaError_t e = cudaGetDevice(&c->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return fail(AF3D_ERR_CUDA, std::string("CUDA unavailable: ") + cudaGetErrorString(e));
  }
  c->own_stream = true;
  c->grid.ntags = ntags;
  const long n = std::max<long>(c->n, 1);
  auto alloc = [&](void **p, size_t bytes) { return cudaMalloc(p, bytes); };
  bool ok = true;
  for (int b = 0; b < 2 && ok; b++) ok = alloc((void **)&c->plane_mem[b], sizeof(double) * n * NPLANES) == cudaSuccess;
  ok = ok && alloc((void **)&c->id_cur, sizeof(long long) * n) == cudaSuccess;
  ok = ok && alloc((void **)&c->id_alt, sizeof(long long) * n) == cudaSuccess;
  ok = ok && alloc((void **)&c->nbr, sizeof(NbrRec) * n) == cudaSuccess;
  ok = ok && alloc((void **)&c->cull, sizeof(CullRec) * n) == cudaSuccess;
  ok = ok && alloc((void **)&c->cells.key, sizeof(int) * n) == cudaSuccess;
  ok = ok && alloc((void **)&c->cells.rank_tmp, sizeof(int) * n) == cudaSuccess;
  ok = ok && alloc((void **)&c->cells.tmp_slot, sizeof(int) * n) == cudaSuccess;
  ok = ok && alloc((void **)&c->cells.perm, sizeof(int) * n) == cudaSuccess;
  ok = ok && alloc((void **)&c->d, sizeof(DevScalars)) == cudaSuccess;
  ok = ok && alloc((void **)&c->d_count, sizeof(unsigned long long)) == cudaSuccess;
  if (!ok) {
    af3d_destroy(c);
    return fail(AF3D_ERR_NOMEM, "device allocation failed");
  }
  for (int k = 0; k < NPLANES; k++) {
    c->cur.p[k] = c->plane_mem[0] + (size_t)k * n;
    c->alt.p[k] = c->plane_mem[1] + (size_t)k * n;
  }
  cudaMemsetAsync(c->plane_mem[0], 0, sizeof(double) * n * NPLANES, c->st);
  cudaMemsetAsync(c->plane_mem[1], 0, sizeof(double) * n * NPLANES, c->st);
  cudaMemsetAsync(c->d, 0, sizeof(DevScalars), c->st);
  cudaMemcpyAsync(&c->d->grid, &c->grid, sizeof(af3d_cell_par), cudaMemcpyHostToDevice, c->st);
  af3d_status s = push_scalars(c);
  if (s) {
    af3d_destroy(c);
    return s;
  }
  *out = c;
  return AF3D_OK;
}

af3d_status af3d_destroy(af3d_ctx *c) {
  if (!c) return AF3D_OK;
  if (c->st) cudaStreamSynchronize(c->st);
  drop_graphs(c);
  for (void *p : {(void *)c->plane_mem[0], (void *)c->plane_mem[1], (void *)c->id_cur, (void *)c->id_alt,
                  (void *)c->nbr, (void *)c->cull, (void *)c->cells.key, (void *)c->cells.rank_tmp,
                  (void *)c->cells.tmp_slot, (void *)c->cells.perm, (void *)c->cells.count,
                  (void *)c->cells.start, (void *)c->cells.block_sums, (void *)c->d, (void *)c->d_aos,
                  (void *)c->d_acc, (void *)c->d_anga, (void *)c->d_tmp, (void *)c->d_count})
    if (p) cudaFree(p);
  if (c->own_stream && c->st) cudaStreamDestroy(c->st);
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
  return push_scalars(c);
}

af3d_status af3d_import_particles(af3d_ctx *c, const af3d_particle *pp, const af3d_vec3 *acc,
                                  const af3d_vec3 *anga) {
  CHECK_CTX(c);
  if (!pp && c->n > 0) return fail(AF3D_ERR_ARG, "null particle array");
  const long n = std::max<long>(c->n, 1);
  if (!c->d_aos) AF3D_CUDA(cudaMalloc(&c->d_aos, sizeof(af3d_particle) * n));
  if (!c->d_acc) AF3D_CUDA(cudaMalloc(&c->d_acc, sizeof(double) * 3 * n));
  if (!c->d_anga) AF3D_CUDA(cudaMalloc(&c->d_anga, sizeof(double) * 3 * n));
  if (c->n > 0) {
    AF3D_CUDA(cudaMemcpyAsync(c->d_aos, pp, sizeof(af3d_particle) * c->n, cudaMemcpyHostToDevice, c->st));
    if (acc) AF3D_CUDA(cudaMemcpyAsync(c->d_acc, acc, sizeof(double) * 3 * c->n, cudaMemcpyHostToDevice, c->st));
    if (anga) AF3D_CUDA(cudaMemcpyAsync(c->d_anga, anga, sizeof(double) * 3 * c->n, cudaMemcpyHostToDevice, c->st));
  }
  launch_aos_to_planes(c->L(), c->d_aos, acc ? c->d_acc : nullptr, anga ? c->d_anga : nullptr, c->cur,
                       c->id_cur);
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  AF3D_CUDA(cudaGetLastError());
  c->imported = true;
  c->records_valid = false;
  c->cells_valid = false;
  drop_graphs(c);
  if (!c->have_grid && c->n > 0) return regrid(c);
  return AF3D_OK;
}

af3d_status af3d_export_particles(af3d_ctx *c, af3d_particle *pp, af3d_vec3 *acc, af3d_vec3 *anga) {
  CHECK_STATE(c);
  if (!pp && c->n > 0) return fail(AF3D_ERR_ARG, "null particle array");
  launch_planes_to_aos(c->L(), c->cur, c->id_cur, c->d_aos, acc ? c->d_acc : nullptr,
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

af3d_status af3d_set_system(af3d_ctx *c, const af3d_system_par *sys) {
  CHECK_CTX(c);
  if (!sys || sys->npart != c->n) return fail(AF3D_ERR_ARG, "system_par npart differs from the context");
  c->sys = *sys;
  return push_scalars(c);
}

af3d_status af3d_get_system(af3d_ctx *c, af3d_system_par *sys) {
  CHECK_CTX(c);
  if (!sys) return fail(AF3D_ERR_ARG, "null argument");
  AF3D_CUDA(cudaMemcpyAsync(&c->sys, &c->d->sys, sizeof(af3d_system_par), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  *sys = c->sys;
  return AF3D_OK;
}

af3d_status af3d_set_grid(af3d_ctx *c, const af3d_cell_par *g) {
  CHECK_CTX(c);
  if (!g || g->ncell.x <= 0 || g->ncell.y <= 0 || g->ncell.z <= 0 ||
      g->ncell3 != g->ncell.x * g->ncell.y * g->ncell.z)
    return fail(AF3D_ERR_ARG, "inconsistent cell_par");
  af3d_cell_par gg = *g;
  gg.ntags = c->ntags;
  return set_grid_device(c, gg);
}

af3d_status af3d_get_grid(af3d_ctx *c, af3d_cell_par *g) {
  CHECK_CTX(c);
  if (!g) return fail(AF3D_ERR_ARG, "null argument");
  AF3D_CUDA(cudaMemcpyAsync(&c->grid, &c->d->grid, sizeof(af3d_cell_par), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  *g = c->grid;
  return AF3D_OK;
}

af3d_status af3d_set_phase(af3d_ctx *c, int phase) {
  CHECK_CTX(c);
  if (phase != AF3D_PHASE_FILL && phase != AF3D_PHASE_AVALANCHE) return fail(AF3D_ERR_ARG, "bad phase");
  af3d_status s = af3d_get_system(c, &c->sys);
  if (s) return s;
  c->phase = phase;
  c->cc = 0;
  return push_scalars(c);
}

af3d_status af3d_regrid(af3d_ctx *c) {
  CHECK_STATE(c);
  c->grid.ntags = c->ntags;
  if (!c->have_grid) {
    af3d_cell_par g{};
    g.ntags = c->ntags;
    AF3D_CUDA(cudaMemcpyAsync(&c->d->grid, &g, sizeof(g), cudaMemcpyHostToDevice, c->st));
  }
  af3d_status s = regrid(c);
  c->cells_valid = false;
  return s;
}

af3d_status af3d_open_door(af3d_ctx *c) {
  CHECK_CTX(c);
  af3d_status s = af3d_get_system(c, &c->sys);
  if (s) return s;
  c->sys.side.x = (70.0 + c->sys.Lflume) * c->sys.cost;   // xfinal, avalanche_hst.cu:116
  c->sys.time = 0.0;
  c->phase = AF3D_PHASE_AVALANCHE;
  c->cc = 0;
  return push_scalars(c);
}

// ---- per-routine entry points ----

af3d_status af3d_init_verlet(af3d_ctx *c) {
  CHECK_STATE(c);
  launch_predict(c->L(), c->cur, c->d, true, false, false, c->cells, c->id_cur);
  c->records_valid = false;
  return AF3D_OK;
}

af3d_status af3d_advance_time(af3d_ctx *c) {
  CHECK_CTX(c);
  launch_advance_time(c->st, c->d);
  c->sys.time = c->sys.time + c->sys.dt;
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
  return AF3D_OK;
}

af3d_status af3d_cell_build(af3d_ctx *c) {
  CHECK_STATE(c);
  if (!c->have_grid) return fail(AF3D_ERR_ARG, "no grid");
  enqueue_cell_build(c, false, false);
  c->records_valid = true;
  c->cells_valid = true;
  return AF3D_OK;
}

af3d_status af3d_force_hop(af3d_ctx *c, int nw) {
  CHECK_STATE(c);
  if (nw < 0 || nw > 2) return fail(AF3D_ERR_ARG, "nw must be 0, 1 or 2");
  launch_boundary(c->L(), c->cur, c->d, R_HOP0 + nw);
  return AF3D_OK;
}

af3d_status af3d_force_funnel(af3d_ctx *c) {
  CHECK_STATE(c);
  launch_boundary(c->L(), c->cur, c->d, R_FUNNEL);
  return AF3D_OK;
}

af3d_status af3d_force_fcorners(af3d_ctx *c) {
  CHECK_STATE(c);
  launch_boundary(c->L(), c->cur, c->d, R_FCORNERS);
  return AF3D_OK;
}

af3d_status af3d_force_walls(af3d_ctx *c) {
  CHECK_STATE(c);
  launch_boundary(c->L(), c->cur, c->d, R_WALLS);
  return AF3D_OK;
}

af3d_status af3d_force_flume(af3d_ctx *c) {
  CHECK_STATE(c);
  launch_boundary(c->L(), c->cur, c->d, R_FLUME);
  return AF3D_OK;
}

af3d_status af3d_force_part(af3d_ctx *c, int sph_id) {
  CHECK_STATE(c);
  if (sph_id < 0 || sph_id > 16) return fail(AF3D_ERR_ARG, "sph_id must be 0..16");
  af3d_status s = ensure_records(c);
  if (s) return s;
  launch_part(c->L(), c->cur, c->d, c->nbr, c->cull, c->cells.start, sph_id);
  return AF3D_OK;
}

af3d_status af3d_get_accel(af3d_ctx *c) {
  CHECK_STATE(c);
  launch_get_accel(c->L(), c->cur, c->d);
  return AF3D_OK;
}

af3d_status af3d_finish_verlet(af3d_ctx *c) {
  CHECK_STATE(c);
  launch_finish_verlet(c->L(), c->cur, c->d);
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
  launch_fused_forces(c->L(), c->cur, c->alt, c->d, c->nbr, c->cull, c->cells.start, true);
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
    for (long i = 0; i < m; i++) c->sys.time = c->sys.time + c->sys.dt;
    const bool do_regrid = (c->cc + m - 1) % kRegridEvery == 0;
    c->cc += m;
    k -= m;
    c->cells_valid = true;
    c->records_valid = false;
    if (do_regrid) {
      s = regrid(c);
      if (s) return s;
      c->cells_valid = false;   // the next step rebuilds the cells on the new grid
    }
  }
  int flags = 0;
  af3d_status s = read_status(c, &flags);
  if (s) return s;
  return first_error(flags);
}

af3d_status af3d_step_profile(af3d_ctx *c, long k, double *ms) {
  CHECK_STATE(c);
  if (k < 0 || !ms) return fail(AF3D_ERR_ARG, "bad argument");
  if (!c->have_grid) return fail(AF3D_ERR_ARG, "no grid");
  cudaEvent_t ev[AF3D_NPROF + 1];
  for (auto &e : ev) AF3D_CUDA(cudaEventCreate(&e));
  for (long i = 0; i < k; i++) {
    AF3D_CUDA(cudaEventRecord(ev[0], c->st));
    launch_advance_time(c->st, c->d);
    AF3D_CUDA(cudaEventRecord(ev[1], c->st));
    launch_predict(c->L(), c->cur, c->d, true, true, true, c->cells, c->id_cur);
    AF3D_CUDA(cudaEventRecord(ev[2], c->st));
    launch_sort(c->L(), c->d, c->cells, c->id_cur, c->ntags);
    AF3D_CUDA(cudaEventRecord(ev[3], c->st));
    launch_permute_records(c->L(), c->cur, c->alt, c->cells.perm, c->id_cur, c->id_alt, c->nbr, c->cull,
                           false);
    std::swap(c->cur, c->alt);
    std::swap(c->id_cur, c->id_alt);
    AF3D_CUDA(cudaEventRecord(ev[4], c->st));
    launch_fused_forces(c->L(), c->cur, c->alt, c->d, c->nbr, c->cull, c->cells.start, false);
    swap_velocity_planes(c->cur, c->alt);
    swap_accel_planes(c->cur);
    swap_accel_planes(c->alt);
    AF3D_CUDA(cudaEventRecord(ev[5], c->st));
    c->launches += kKernelsPerStep;
    c->sys.time = c->sys.time + c->sys.dt;
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
  }
  for (auto &e : ev) cudaEventDestroy(e);
  c->cells_valid = c->cc % kRegridEvery != 1;
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
  // Reuse the export path's id scatter through a temporary AoS-free copy.
  std::vector<double> hp(6 * (size_t)c->n);
  std::vector<long long> ids((size_t)c->n);
  if (c->n == 0) return AF3D_OK;
  for (int k = 0; k < 6; k++)
    AF3D_CUDA(cudaMemcpyAsync(hp.data() + (size_t)k * c->n, c->cur.p[FX + k], sizeof(double) * c->n,
                              cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaMemcpyAsync(ids.data(), c->id_cur, sizeof(long long) * c->n, cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  for (long s = 0; s < c->n; s++) {
    const long long i = ids[s];
    if (force) force[i] = {hp[s], hp[c->n + s], hp[2 * c->n + s]};
    if (torque) torque[i] = {hp[3 * c->n + s], hp[4 * c->n + s], hp[5 * c->n + s]};
  }
  return AF3D_OK;
}

af3d_status af3d_get_accels(af3d_ctx *c, af3d_vec3 *acc_f, af3d_vec3 *anga_f) {
  CHECK_STATE(c);
  std::vector<double> hp(6 * (size_t)c->n);
  std::vector<long long> ids((size_t)c->n);
  if (c->n == 0) return AF3D_OK;
  for (int k = 0; k < 6; k++)
    AF3D_CUDA(cudaMemcpyAsync(hp.data() + (size_t)k * c->n, c->cur.p[AFX + k], sizeof(double) * c->n,
                              cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaMemcpyAsync(ids.data(), c->id_cur, sizeof(long long) * c->n, cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  for (long s = 0; s < c->n; s++) {
    const long long i = ids[s];
    if (acc_f) acc_f[i] = {hp[s], hp[c->n + s], hp[2 * c->n + s]};
    if (anga_f) anga_f[i] = {hp[3 * c->n + s], hp[4 * c->n + s], hp[5 * c->n + s]};
  }
  return AF3D_OK;
}

af3d_status af3d_get_cells(af3d_ctx *c, long *cell_of_id, long *sorted_ids, long *nbinned) {
  CHECK_STATE(c);
  if (!c->cells_valid) return fail(AF3D_ERR_ARG, "no cell build since the last grid change");
  if (c->n == 0) {
    if (nbinned) *nbinned = 0;
    return AF3D_OK;
  }
  if (!c->d_tmp) AF3D_CUDA(cudaMalloc(&c->d_tmp, sizeof(long long) * c->n));
  af3d_cell_par g;
  AF3D_CUDA(cudaMemcpyAsync(&g, &c->d->grid, sizeof(g), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  int nb = 0;
  AF3D_CUDA(cudaMemcpy(&nb, c->cells.start + g.ncell3, sizeof(int), cudaMemcpyDeviceToHost));
  if (nbinned) *nbinned = nb;
  if (cell_of_id) {
    // keys belong to the layout before the last permutation, whose ids are now in id_alt
    launch_cells_by_id(c->L(), c->cells.key, c->id_alt, g.ncell3, c->d_tmp);
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
  long long *d_out = nullptr;
  if (cap > 0) AF3D_CUDA(cudaMalloc(&d_out, sizeof(long long) * 3 * cap));
  AF3D_CUDA(cudaMemsetAsync(c->d_count, 0, sizeof(unsigned long long), c->st));
  launch_contact_pairs(c->L(), c->cur, c->d, c->nbr, c->cull, c->cells.start, c->id_cur, d_out, c->d_count,
                       cap, active);
  unsigned long long cnt = 0;
  AF3D_CUDA(cudaMemcpyAsync(&cnt, c->d_count, sizeof(cnt), cudaMemcpyDeviceToHost, c->st));
  AF3D_CUDA(cudaStreamSynchronize(c->st));
  if (count) *count = (long)cnt;
  if (cap > 0 && out)
    AF3D_CUDA(cudaMemcpy(out, d_out, sizeof(long long) * 3 * std::min<long>(cap, (long)cnt),
                         cudaMemcpyDeviceToHost));
  if (d_out) cudaFree(d_out);
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

}  // extern "C"
