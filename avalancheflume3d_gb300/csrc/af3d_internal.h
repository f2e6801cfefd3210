// af3d_internal.h -- definitions shared by the device kernels and the host side of the C ABI.
//
// Device state layout (HBM): every per-clump scalar is one FP64 "plane" of length N, in the
// (cell, id)-sorted order of the last cell build.  The cell build permutes every plane, so the
// clumps of one cell -- and of neighbouring cells along x -- sit in consecutive slots and all
// per-clump kernels read and write coalesced.  Two plane sets (cur / alt) are ping-ponged by the
// permutation.  Neighbour-visible data is additionally packed per slot into an FP64 record
// (NbrRec, 192 B) and an FP32 culling record (CullRec, 80 B) so that a neighbour gather touches
// one or two 64-byte lines.
#pragma once

#include <cstdint>
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "../../include/af3d.h"

namespace af3d {

enum Plane : int {
  RX, RY, RZ, VX, VY, VZ, WX, WY, WZ,
  R00, R01, R02, R10, R11, R12, R20, R21, R22,   // Rmatx, Rmaty, Rmatz rows
  AIX, AIY, AIZ, ALIX, ALIY, ALIZ,               // a_i, alpha_i
  AFX, AFY, AFZ, ALFX, ALFY, ALFZ,               // a_f, alpha_f
  S0X, S0Y, S0Z, S1X, S1Y, S1Z, S2X, S2Y, S2Z, S3X, S3Y, S3Z,   // sphere centres rr_a..rr_d
  FX, FY, FZ, TX, TY, TZ,                        // force, torque accumulators
  RAD, DEN, MASS, IXX, IYY, IZZ,                 // radius, density, clump mass, inertia
  MSPH,                                          // SPH_FACT*density*r^3 (force_part.cu:58 order)
  MWALL,                                         // SPH_FACT*r^3*density (force_walls.cu:47 order)
  ADRAG,                                         // DRAG*r*r/mass (get_accel.cu:47 order)
  IMASS, IINER,                                  // 1/mass, 1/inertia (fast FP64 mode)
  RN00, RN01, RN02, RN10, RN11, RN12, RN20, RN21, RN22,   // next step's rotation rows (look-ahead)
  NPLANES
};

struct Planes {
  double *p[NPLANES];
};

// Packed neighbour record: everything a partner clump contributes to a contact.
struct __align__(64) NbrRec {
  double rx, ry, rz, vx, vy, vz, wx, wy, wz;
  double s[12];          // sphere k: s[3k], s[3k+1], s[3k+2]
  double rad, msph, mwall;   // sphere radius, sphere mass, wall-contact mass
};

// FP32 culling record.  c = (centre, bound), sk = (sphere centre, inflated radius).  The bounds
// are rounded up and inflated by 2^-22 times the largest coordinate magnitude, which covers the
// FP32 rounding of every coordinate; the tests multiply by (1 + 2^-18) on top, so a pair the
// FP64 test could accept is never culled.
struct __align__(16) CullRec {
  float4 c;
  float4 s[4];
};

// Cell-list buffers.  Keys: flume cell offset + cell index for binned clumps (the flumes' grids
// are concatenated, so the sort keeps every flume contiguous), ncell_total + id for clumps that
// are not binned (removed), so every bucket holds its clumps in id order after the rank pass and
// no bucket is large.
struct Cells {
  int *key;         // [N]   key of old slot
  int *rank_tmp;    // [N]   atomic arrival rank inside the bucket (nondeterministic)
  int *tmp_slot;    // [N]   old slots scattered by arrival order
  int *perm;        // [N]   new slot -> old slot, deterministic (cell, id) order
  float4 *csort;    // [N]   FP32 culling centre of the clump at each position of that order
  int *count;       // [cap] bucket sizes (all zero between builds)
  int *start;       // [cap+1] exclusive scan of count
  int *tile_count;  // [scan_tiles(cap)] clumps per kScanTile buckets (all zero between builds)
  long cap;         // buckets available (ncell_total + N must fit)
};

// Buckets per tile of the sort's scan.
constexpr int kScanTile = 4096;

// A clump's arrival in bucket `key`: returns its rank among the bucket's arrivals, and counts it
// in the key's scan tile too, so that the sort's scan starts from the tile counts instead of
// summing every bucket in a pass of its own.  A warp's clumps lie mostly in one tile (slots are
// in spatial order), so the lanes arriving together add to each tile once: one atomic per
// distinct tile instead of one per clump, which contended on the tile's counter.
__device__ __forceinline__ int arrive_in_bucket(const Cells &c, long key) {
  namespace cg = cooperative_groups;
  const int tile = (int)(key / kScanTile);
  const cg::coalesced_group here = cg::coalesced_threads();
  const cg::coalesced_group same = cg::labeled_partition(here, tile);
  if (same.thread_rank() == 0) atomicAdd(&c.tile_count[tile], (int)same.size());
  return atomicAdd(&c.count[key], 1);
}

// Scalars of one flume's system_par / Funnel used by the force routines.  A single-flume
// context passes them to the fused force kernel as a __grid_constant__ parameter (constant-bank
// operands, no registers held); the clock is read through `tp` (it advances on the device).
struct Consts {
  double dt, hdt;
  double mu_pp, kappa_pp, gamma_pp, cns_pp;
  double mu_pw, kappa_pw, gamma_pw, cns_pw;
  double sint, cost, dy2, side_x, side_y;
  double sinfi, cosfi, tanfi;
  double tant;     // sint / cost
  double inv_dt;   // 1 / dt (fast mode)
  double qk_pp, qg_pp, hk_pw, hg_pw;   // kappa_pp / 4, gamma_pp / 4, kappa_pw / 2, gamma_pw / 2 (fast mode)
  const double *tp;   // the device clock, DevScalars::time
  float cost_f, sint_f, tanfi_f, cosfi_f, dy2_f, side_y_f;   // FP32 copies for the culling gates
  int phase, variant;
};

// The constants of a flume from its parameters (the same values the device loads).
__host__ __device__ inline Consts make_consts(const af3d_system_par &s, const af3d_funnel &fun, double tant, int phase, int variant,
                          const double *tp) {
  Consts c;
  c.dt = s.dt; c.hdt = s.hdt;
  c.mu_pp = s.mu_pp; c.kappa_pp = s.kappa_pp; c.gamma_pp = s.gamma_pp; c.cns_pp = s.fr_fact_pp;
  c.mu_pw = s.mu_pw; c.kappa_pw = s.kappa_pw; c.gamma_pw = s.gamma_pw; c.cns_pw = s.fr_fact_pw;
  c.sint = s.sint; c.cost = s.cost; c.dy2 = s.dy2; c.side_x = s.side.x; c.side_y = s.side.y;
  c.sinfi = fun.sinfi; c.cosfi = fun.cosfi; c.tanfi = fun.tanfi;
  c.tant = tant;
  c.inv_dt = 1.0 / s.dt;
  c.qk_pp = 0.25 * s.kappa_pp; c.qg_pp = 0.25 * s.gamma_pp;
  c.hk_pw = 0.5 * s.kappa_pw; c.hg_pw = 0.5 * s.gamma_pw;
  c.tp = tp;
  c.cost_f = (float)s.cost; c.sint_f = (float)s.sint; c.tanfi_f = (float)fun.tanfi; c.cosfi_f = (float)fun.cosfi;
  c.dy2_f = (float)s.dy2; c.side_y_f = (float)s.side.y;
  c.phase = phase; c.variant = variant;
  return c;
}

// One flume of the context (a plain drop-in run has one; a batched ensemble has many).  Every
// flume has its own system_par (friction, restitution, slope, ...), Funnel and cell grid; all
// flumes share dt and advance in lockstep.
// FP32 copies of a grid's origin and inverse cell sides (the search-cell estimate).
struct GridF {
  float xmin, ymin, zmin, ix, iy, iz;
};

__host__ __device__ inline GridF grid_floats(const af3d_cell_par &g) {
  GridF q;
  q.xmin = (float)g.rr_min.x; q.ymin = (float)g.rr_min.y; q.zmin = (float)g.rr_min.z;
  q.ix = (float)g.cs_inv.x; q.iy = (float)g.cs_inv.y; q.iz = (float)g.cs_inv.z;
  return q;
}

struct DevFlume {
  af3d_system_par sys;        // sys.time is unused: the shared clock is DevScalars::time
  af3d_funnel     fun;
  af3d_cell_par   grid;
  GridF           gridf;      // grid_floats(grid), written with it
  long long       cell_off;   // first bucket of this flume's cells
  double          tant;       // sys.sint / sys.cost (force_flume.cu's tangent), set by the host
  unsigned long long bbox[8]; // re-grid scratch: ordered-int min/max of x, y, z, max vx, min vz
  af3d_cell_par   pending;    // grid derived by the last re-grid, committed when it fits
  Consts          c;          // make_consts of sys, fun, tant and the context's phase/variant
};

// Per-context device scalars (one struct in global memory).
struct DevScalars {
  double          time;       // current time (after the last advance)
  double          time_prev;  // time before the last advance (init_Verlet's removal test)
  int             phase;      // AF3D_PHASE_*
  int             variant;    // AF3D_FRICTION_*
  int             status;     // bitmask of 1 << AF3D_ERR_*
  int             nflumes;
  unsigned long long contacts; // active sphere-sphere contacts summed over fused force passes
  unsigned long long overflows; // clumps whose item lists overflowed, over fused force passes
  long long       ncell_total; // sum of the flumes' ncell3: the first removed-clump bucket
  long long       pending;     // > 0: a re-grid derived grids needing this many cell buckets
  DevFlume       *flumes;      // [nflumes]
};

// Shapes of the fused force kernel: threads per block (the pool of clumps whose contact items a
// block processes together) and resident blocks per SM (the register budget, 65536 / (block x
// blocks)).  Results do not depend on the shape; af3d_autotune_shapes times them, and a new
// context starts with the default shape whose last wave of blocks is fullest on its device
// (force_shape_for).  192 x 3 is tuned but not a default: its larger pool wastes fewer lanes in
// the last round of contact laws, which pays in the exact mode's heavier law, but at a few
// blocks per SM it spreads small counts over fewer SMs.
constexpr int kForceShapes = 4;
constexpr int kForceShapeBlock[kForceShapes] = {128, 96, 64, 192};
constexpr int kForceShapeMinb[kForceShapes] = {5, 6, 10, 3};
constexpr bool kForceShapeDefault[kForceShapes] = {true, true, true, false};
// Steps whose force pass runs in parts (af3d_step_host) cut the clumps at multiples of every
// shape's block.
constexpr long kForceAlign = 384;
static_assert(kForceAlign % 128 == 0 && kForceAlign % 96 == 0 && kForceAlign % 64 == 0 && kForceAlign % 192 == 0,
              "a multiple of every shape's block");

// Per-clump item lists of one force pass, from the list phase to the force phase of the force
// kernel: entry e of slot s at items[e * n + s] (an item is a boundary (routine, sphere) or a
// particle (partner slot, sph_id) contact).  With cnt, the pass also records each clump's list
// layout there (pack_list_counts), which lets the adjoint reverse the pass from the same lists,
// and with ovf sets *ovf when any clump's lists overflowed (its contacts then ran by the
// per-clump walk, which needs the pass's cell structure).
constexpr int kListCap = 32;
struct ContactLists {
  unsigned *items;   // [kListCap][n]
  int *cnt;          // [n] or null
  int *ovf;          // or null
};

// A clump's list layout as one int: -1 when its lists overflowed, else the item count | the
// boundary items before the particle items << 8 | the particle items << 16 (each at most 32).
__host__ __device__ inline int pack_list_counts(int listed, int pre, int pair) {
  return listed < 0 ? -1 : listed | pre << 8 | pair << 16;
}

// The next step's predictor run at the end of a force pass (look-ahead): the corrected clump is
// advanced at once, its records go to the next step's record buffers, its rotation rows to the
// RN planes, its bucket key, arrival rank and bucket count to the cell list.  nbr == null: none.
struct LookAhead {
  NbrRec *nbr;
  CullRec *cull;
  Cells cells;
  const long long *id;
};

// Which force routines a boundary kernel applies, in the reference's call order.
enum Routine : int {
  R_HOP0 = 0, R_HOP1, R_HOP2, R_FUNNEL, R_FCORNERS, R_WALLS, R_FLUME
};

// ---- kernel launchers (defined in the .cu files; all enqueue on `st`) ----
struct Launch {
  cudaStream_t st;
  long n;
};

// init_Verlet and/or the cell keys; with nbr/cull (predict and keys only) also the neighbour
// records of every clump at its own slot.
void launch_predict (const Launch &L, Planes cur, DevScalars *d, bool predict, bool keys, bool t_prev,
                     Cells cells, const long long *id, const int *flume, NbrRec *nbr = nullptr,
                     CullRec *cull = nullptr, long s0 = 0, long count = -1);
// Exclusive scan of the bucket counts, scatter by arrival, then the deterministic (bucket, id)
// rank: fills cells.start[0..nbuckets] and cells.perm, checks the ntags capacity and leaves the
// count array zeroed.  nbuckets = ncell_total + N is read on the device.
// With cull (records already written at the old slots) also fills cells.csort.
void launch_sort (const Launch &L, DevScalars *d, Cells cells, const long long *id, long ntags,
                  const CullRec *cull = nullptr, bool advance = false);
long scan_tiles (long bucket_cap);
// Moves every plane (and the id and flume arrays) into the new order and builds the records.
// `ft`: also carry the force/torque accumulators and a_f (the fused step rewrites them first).
void launch_permute_records (const Launch &L, Planes src, Planes dst, const int *perm,
                             const long long *id_src, long long *id_dst, const int *fl_src,
                             int *fl_dst, NbrRec *nbr, CullRec *cull, bool ft);
void launch_build_records (const Launch &L, Planes cur, NbrRec *nbr, CullRec *cull);
// The force pass: each block builds its clumps' item lists, then processes them (walls, contacts,
// bed, get_accel, finish_Verlet).  order: null when the slots are in (cell, id) order, else
// cells.perm of the last sort, with csort the matching culling centres.  warm: the step's
// predicted state was made by the previous pass's look-ahead (records, RN planes) and is
// committed to the planes here; look: this pass runs the next step's predictor.
void launch_lists_forces (const Launch &L, Planes cur, Planes out, DevScalars *d, const int *flume,
                          const NbrRec *nbr, const CullRec *cull, const int *start, const int *order,
                          const float4 *csort, ContactLists lists, bool write_ft,
                          const Consts *uniform = nullptr, bool warm = false,
                          LookAhead look = LookAhead{}, long s0 = 0, long count = -1, int shape = 0);
void launch_boundary (const Launch &L, Planes cur, DevScalars *d, const int *flume, int routine);
void launch_part (const Launch &L, Planes cur, DevScalars *d, const int *flume, const NbrRec *nbr,
                  const CullRec *cull, const int *start, int sph_id);
void launch_get_accel (const Launch &L, Planes cur, DevScalars *d, const int *flume);
void launch_finish_verlet (const Launch &L, Planes cur, DevScalars *d, const int *flume);
void launch_clear_forces (const Launch &L, Planes cur);
void launch_advance_time (cudaStream_t st, DevScalars *d);
// Per-flume cell_dim + grid derivation; commits the grids (and bucket offsets) when they fit
// bucket_cap, else leaves them pending (DevScalars::pending = buckets needed).
void launch_regrid (const Launch &L, Planes cur, DevScalars *d, const int *flume, int nflumes,
                    long bucket_cap);
// Re-commit pending grids after the host grew the bucket buffers.
void launch_commit_grids (cudaStream_t st, DevScalars *d, int nflumes, long n, long bucket_cap);
// AoS particles (+ a_i, alpha_i) into the planes, clump id at slot id for the first import
// (keep_order false), else at the slot the clump already holds (the slot order is kept).
void launch_aos_to_planes (const Launch &L, const af3d_particle *aos, const double *acc,
                           const double *anga, const int *flume_of_id, Planes cur, long long *id,
                           int *flume, bool keep_order, long s0 = 0, long count = -1);
void launch_planes_to_aos (const Launch &L, Planes cur, const long long *id, const int *flume,
                           af3d_particle *aos, double *acc, double *anga, DevScalars *d, long s0 = 0,
                           long count = -1);
void launch_contact_pairs (const Launch &L, Planes cur, DevScalars *d, const int *flume,
                           const NbrRec *nbr, const CullRec *cull, const int *start,
                           const long long *id, long long *out, unsigned long long *count, long cap,
                           int active);
void launch_cells_by_id (const Launch &L, const int *key, const long long *id, DevScalars *d,
                         long long *cell_of_id);
// DFMA throughput microbenchmark (TFLOP/s, 2 flops per DFMA), bounded to ~0.1 s.
cudaError_t measure_dfma (int sms, double *tflops);
// Per element of x, a bit for each integer-pipe FP64 helper that disagrees with the hardware.
cudaError_t check_fp64_bits (const double *x, long n, int *bad);

// Adjoint of the exact step (af3d_adjoint.cu).  Planes of 24 state adjoints (r, v, w, R rows,
// a_i, alpha_i), 21 scattered parts (r1, v1, w1, sphere centres), 9 own R1 parts.
constexpr int kAdjPlanes = 24, kAccPlanes = 21, kRbPlanes = 9;
void launch_adj_forces (const Launch &L, Planes P, Planes in, Planes out, Planes acc, Planes rb, DevScalars *d,
                        const int *flume, const NbrRec *nbr, const CullRec *cull, const int *start,
                        const int *order, const float4 *csort, double *param_b, bool startup);
// The same reverse (not the start-up pass) from the item lists and counts the forward force pass
// of this step recorded.
void launch_adj_forces_lists (const Launch &L, Planes P, Planes in, Planes out, Planes acc, Planes rb,
                              DevScalars *d, const int *flume, const NbrRec *nbr, const CullRec *cull,
                              const int *start, const int *order, ContactLists lists, double *param_b);
void launch_adj_predict (const Launch &L, Planes P, Planes tape, Planes in, Planes out, Planes acc, Planes rb,
                         DevScalars *d, const int *flume);
void launch_adj_startup (const Launch &L, Planes P, Planes in, Planes out, Planes acc, Planes rb);
// Objective sums (3 per flume, zeroed before) and the adjoint seed of the final state; length
// > 0: the runout soft maximum with that length scale, else the deposit centroid.
void launch_adj_objective (const Launch &L, Planes P, DevScalars *d, const int *flume, double *sums, double length);
void launch_adj_seed (const Launch &L, Planes P, Planes adj, DevScalars *d, const int *flume, const double *sums,
                      double length);
// The 24 state planes (with spheres: 36, the sphere centres too) between the plane set and a
// tape slot (to_tape: planes -> tape).
void launch_state_copy (const Launch &L, Planes P, Planes tape, bool to_tape, bool spheres = false);

// The predictor and the fused force pass of the fast FP64 mode (af3d_kernels.cu compiled with
// -DAF3D_FAST -fmad=true; same arguments as above).
namespace fast {
void launch_predict (const Launch &L, Planes cur, DevScalars *d, bool predict, bool keys, bool t_prev,
                     Cells cells, const long long *id, const int *flume, NbrRec *nbr = nullptr,
                     CullRec *cull = nullptr, long s0 = 0, long count = -1);
void launch_lists_forces (const Launch &L, Planes cur, Planes out, DevScalars *d, const int *flume,
                          const NbrRec *nbr, const CullRec *cull, const int *start, const int *order,
                          const float4 *csort, ContactLists lists, bool write_ft,
                          const Consts *uniform = nullptr, bool warm = false,
                          LookAhead look = LookAhead{}, long s0 = 0, long count = -1, int shape = 0);
}  // namespace fast

}  // namespace af3d
