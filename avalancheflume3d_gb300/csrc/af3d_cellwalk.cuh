// af3d_cellwalk.cuh -- the FP32 culling tests and the neighbour-cell walk of the sorted cell
// list, shared by the step kernels and the adjoint kernels.
#pragma once

#include "af3d_physics.cuh"

namespace af3d {
namespace {

constexpr float kCullSlack = 1.0f + 3.814697265625e-06f;  // 1 + 2^-18

// Squared distance for the conservative FP32 culling tests (fused multiply-adds: their rounding
// error is below the unfused one, and the tests' 2^-18 slack covers either).
__device__ __forceinline__ float d2f(float4 a, float4 b) {
  const float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
  return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// 16-bit mask of the sphere pairs of own clump (cull record me) and partner m that the FP32
// test cannot rule out; bit p = sph_id - 1 = 4 * (partner sphere) + (own sphere).
__device__ __forceinline__ unsigned pair_mask(const CullRec &me, const CullRec &m) {
  const float lim = me.c.w + m.c.w;
  if (d2f(me.c, m.c) > lim * lim * kCullSlack) return 0u;
  const float rl = me.s[0].w + m.s[0].w;
  const float r2 = rl * rl * kCullSlack;
  unsigned mask = 0u;
#pragma unroll
  for (int j = 0; j < 4; j++)
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (d2f(me.s[k], m.s[j]) <= r2) mask |= 1u << (4 * j + k);
  return mask;
}

// The sixteen sphere tests of pair_mask alone (for partners whose centre test passed).
__device__ __forceinline__ unsigned sphere_mask(const CullRec &me, const CullRec &m) {
  const float rl = me.s[0].w + m.s[0].w;
  const float r2 = rl * rl * kCullSlack;
  unsigned mask = 0u;
#pragma unroll
  for (int j = 0; j < 4; j++)
#pragma unroll
    for (int k = 0; k < 4; k++)
      if (d2f(me.s[k], m.s[j]) <= r2) mask |= 1u << (4 * j + k);
  return mask;
}

struct Search {
  long ci, cj, ck;
  long long off;   // the flume's first cell bucket
};

// Search-centre cell of force_part.cu:77-85: (long)((x - xmin)/side).  The quotient is first
// estimated with the reciprocal cs_inv = 1/side.  For |q| < 1e6 the estimate is within
// 4.4e-16 |Q| < 1e-9 of the true quotient Q, so when it is more than 1e-9 away from an integer,
// Q and its correctly rounded value lie in the same open unit interval and truncate to the same
// index; the division is only carried out near a cell boundary.  Same index as the reference.
__device__ __forceinline__ long search_axis(double x, double xmin, double side, double inv, long n) {
  const double dx = x - xmin;
  const double q = dx * inv;
  const double fl = floor(q);
  long i;
  if (q - fl > 1e-9 && q - fl < 1.0 - 1e-9 && fabs(q) < 1.0e6)   // |q - Q| <= 4.4e-16 |Q| < 1e-9
    i = (long)q;
  else
    i = (long)(dx / side);
  if (i == n) i--;
  return i;
}

__device__ __forceinline__ Search search_centre(V3 r, const af3d_cell_par &g, long long off) {
  Search q;
  q.off = off;
  q.ci = search_axis(r.x, g.rr_min.x, g.cell_side.x, g.cs_inv.x, g.ncell.x);
  q.cj = search_axis(r.y, g.rr_min.y, g.cell_side.y, g.cs_inv.y, g.ncell.y);
  q.ck = search_axis(r.z, g.rr_min.z, g.cell_side.z, g.cs_inv.z, g.ncell.z);
  return q;
}

// Visit the occupied slots of the 27 neighbour cells in the reference's order
// (idel, jdel, kdel from -1 to 1; force_part.cu:88-106); slots inside a cell are in id order.
// `order` (may be null): the slot of the clump at each position of the (cell, id) order, for
// steps that do not move the clumps into that order.
template <typename F>
__device__ __forceinline__ void for_neighbour_slots(const Search &q, const af3d_cell_par &g,
                                                    const int *__restrict__ start,
                                                    const int *__restrict__ order, F &&f) {
#pragma unroll 1
  for (int di = -1; di <= 1; di++)
#pragma unroll 1
    for (int dj = -1; dj <= 1; dj++)
#pragma unroll 1
      for (int dk = -1; dk <= 1; dk++) {
        const long in = q.ci + di, jn = q.cj + dj, kn = q.ck + dk;
        if (in < 0 || jn < 0 || kn < 0 || in >= g.ncell.x || jn >= g.ncell.y || kn >= g.ncell.z)
          continue;
        const long c = q.off + in + g.ncell.x * (jn + g.ncell.y * kn);
        const int t0 = __ldg(&start[c]), t1 = __ldg(&start[c + 1]);
#pragma unroll 1
        for (int t = t0; t < t1; t++) f(order ? __ldg(&order[t]) : t);
      }
}

// The positions (in the (cell, id) order) of the 27 neighbour cells' clumps, in the reference's
// order, with every cell boundary loaded up front (as below).
template <typename F>
__device__ __forceinline__ void for_neighbour_positions_pre(const Search &q, const af3d_cell_par &g,
                                                            const int *__restrict__ start, F &&f) {
  int bnd[9][4];
  const long x0 = q.ci - 1;
#pragma unroll
  for (int r = 0; r < 9; r++) {
    const long jn = q.cj + (r / 3 - 1), kn = q.ck + (r % 3 - 1);
    const bool row_ok = jn >= 0 && kn >= 0 && jn < g.ncell.y && kn < g.ncell.z;
    const long rb = q.off + g.ncell.x * (jn + g.ncell.y * kn);
#pragma unroll
    for (int e = 0; e < 4; e++) {
      long x = x0 + e;
      x = x < 0 ? 0 : (x > g.ncell.x ? g.ncell.x : x);
      bnd[r][e] = row_ok ? __ldg(&start[rb + x]) : 0;
    }
  }
#pragma unroll 1
  for (int di = 0; di < 3; di++)
#pragma unroll 1
    for (int r = 0; r < 9; r++) {
      const int k0 = bnd[r][di], k1 = bnd[r][di + 1];
#pragma unroll 1
      for (int k = k0; k < k1; k++) f(k);
    }
}

// The same visit with every cell boundary loaded up front.  The three cells of one (jdel, kdel)
// row are consecutive in the linear cell index, so their members form one slot range split by
// four start[] values; the 9 rows x 4 boundaries are issued as independent loads before the walk
// (instead of 27 dependent round trips), then the cells are walked in the reference's order.
template <typename F>
__device__ __forceinline__ void for_neighbour_slots_pre(const Search &q, const af3d_cell_par &g,
                                                        const int *__restrict__ start,
                                                        const int *__restrict__ order, F &&f) {
  int bnd[9][4];
  const long x0 = q.ci - 1;
#pragma unroll
  for (int r = 0; r < 9; r++) {
    const long jn = q.cj + (r / 3 - 1), kn = q.ck + (r % 3 - 1);
    const bool row_ok = jn >= 0 && kn >= 0 && jn < g.ncell.y && kn < g.ncell.z;
    const long rb = q.off + g.ncell.x * (jn + g.ncell.y * kn);
#pragma unroll
    for (int e = 0; e < 4; e++) {
      // boundary e of the row: start of cell x0 + e, clamped into the row (empty cells outside)
      long x = x0 + e;
      x = x < 0 ? 0 : (x > g.ncell.x ? g.ncell.x : x);
      bnd[r][e] = row_ok ? __ldg(&start[rb + x]) : 0;
    }
  }
#pragma unroll 1
  for (int di = 0; di < 3; di++)
#pragma unroll 1
    for (int r = 0; r < 9; r++) {
      const int t0 = bnd[r][di], t1 = bnd[r][di + 1];
#pragma unroll 1
      for (int t = t0; t < t1; t++) f(order ? __ldg(&order[t]) : t);
    }
}

// ---- per-warp item lists (the warp-cooperative contact passes) -----------------------------

constexpr int kLaneItems = 32;
constexpr unsigned kBndItem = 0xFFFFFF00u;   // boundary item: kBndItem | routine << 2 | sphere

constexpr int kPassCap = 32;   // partners per clump that pass the centre test

// Per-warp item lists in shared memory, one column per lane ([entry][lane]): a lane's own
// accesses always fall in its own bank, whatever entry each lane is at.
struct ItemLists {
  unsigned items[kLaneItems][32];
  int base[33];                          // exclusive prefix of the lanes' item counts
  int pass_t[kPassCap][32];              // partner slots in walk order, per lane
  unsigned short pass_m[kPassCap][32];   // their 16-bit sphere-pair masks
  int pbase[33];
};

// Exclusive prefix of `v` over the warp into sh[0..32]; returns the total.
__device__ __forceinline__ int warp_prefix(int v, int *sh) {
  const int lane = threadIdx.x & 31;
  int incl = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += u;
  }
  sh[lane] = incl - v;
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  if (lane == 31) sh[32] = total;
  __syncwarp();
  return total;
}

// The lane whose range [sh[l], sh[l+1]) holds position j (sh: exclusive prefix of 32 counts).
__device__ __forceinline__ int owner_of(const int *sh, int j) {
  int lo = 0, hi = 31;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (sh[mid] <= j) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Boundary items of the routines [r0, r1] for one clump (appended to the lane's column `col`,
// entry stride 32); false if the list would overflow.
__device__ __forceinline__ bool push_boundary(int r0, int r1, const Own &o, double B, const Consts &c,
                                              unsigned *col, int &nitems) {
  for (int rt = r0; rt <= r1; rt++) {
    if (!bnd_may_touch(rt, o.r, B, c)) continue;
    for (int ns = 0; ns < 4; ns++) {
      if (!bnd_may_touch(rt, o.s[ns], o.rad, c)) continue;   // the gate applied to one sphere
      if (nitems == kLaneItems) return false;
      col[32 * nitems++] = kBndItem | (unsigned)(rt << 2) | (unsigned)ns;
    }
  }
  return true;
}

// Every lane's item list of one contact pass, in the reference's order: the boundary routines
// before the particles (avalanche: hop x3, funnel, fcorners, walls), the particle contacts
// sph_id-major, the routines after them (avalanche: flume; fill: hop x3).  Boundary items
// (routine, sphere) for the spheres the routine's 1-Lipschitz gate cannot rule out; particle
// items (partner slot, sph_id) from a two-stage gather: stage 1 (per lane) walks the 27
// neighbour cells keeping the partners whose bounding spheres can touch, stage 2 (whole warp)
// runs the sixteen sphere tests of every kept partner, 32 a round.  All 32 lanes call this;
// returns the lane's item count, 0 with `slow` set when the lane's lists would overflow.
__device__ __forceinline__ int build_item_lists(ItemLists &il, long wbase, long s, bool act, bool aval, double B,
                                                const Own &o, const Consts &c, const af3d_cell_par &g,
                                                long long off, const CullRec *__restrict__ cull,
                                                const int *__restrict__ start, const int *__restrict__ order,
                                                const float4 *__restrict__ csort, bool &slow) {
  const int lane = threadIdx.x & 31;
  const int pre0 = aval ? R_HOP0 : 1, pre1 = aval ? R_WALLS : 0;         // fill: none before
  const int post0 = aval ? R_FLUME : R_HOP0, post1 = aval ? R_FLUME : R_HOP2;
  int nitems = 0;
  slow = false;
  unsigned *L = &il.items[0][lane];   // the lane's column
  if (act) slow = !push_boundary(pre0, pre1, o, B, c, L, nitems);
  // Particle partners, stage 1 (per lane): walk the 27 neighbour cells in the reference's order
  // and keep the partners whose bounding spheres can touch (FP32 centre test).
  int npass = 0;
  if (act && !slow) {
    const float4 mc = cull[s].c;
    const Search q = search_centre(o.r, g, off);
    for_neighbour_positions_pre(q, g, start, [&](int k) {
      // the culling centre at position k: contiguous along a cell row in either layout
      const float4 pc = order ? __ldg(&csort[k]) : cull[k].c;
      const float lim = mc.w + pc.w;
      if (d2f(mc, pc) > lim * lim * kCullSlack) return;
      const int t = order ? __ldg(&order[k]) : k;
      if (t == s) return;
      if (npass < kPassCap) il.pass_t[npass][lane] = t;
      npass++;
    });
    if (npass > kPassCap) {
      slow = true;
      npass = 0;
    }
  }
  // Stage 2 (whole warp): the sixteen sphere tests of every kept partner, 32 partners a round.
  const int total_pass = warp_prefix(npass, il.pbase);
  for (int j0 = 0; j0 < total_pass; j0 += 32) {
    const int j = j0 + lane;
    if (j < total_pass) {
      const int ow = owner_of(il.pbase, j), k = j - il.pbase[ow];
      il.pass_m[k][ow] = (unsigned short)sphere_mask(cull[wbase + ow], cull[il.pass_t[k][ow]]);
    }
  }
  __syncwarp();
  // Each lane's particle items, sph_id-major (the order of the sixteen force_part launches):
  // the partners without a candidate sphere pair are dropped first (keeping the walk order), and
  // only the sph_ids some partner has are visited.
  if (act && !slow) {
    int m = 0;
    unsigned any = 0u;
#pragma unroll 1
    for (int k = 0; k < npass; k++) {
      const unsigned mk16 = il.pass_m[k][lane];
      if (!mk16) continue;
      il.pass_t[m][lane] = il.pass_t[k][lane];
      il.pass_m[m][lane] = (unsigned short)mk16;
      any |= mk16;
      m++;
    }
#pragma unroll 1
    while (any && !slow) {
      const int p = __ffs(any) - 1;
      any &= any - 1u;
#pragma unroll 1
      for (int k = 0; k < m; k++) {
        if (!((il.pass_m[k][lane] >> p) & 1u)) continue;
        if (nitems == kLaneItems) {
          slow = true;
          break;
        }
        L[32 * nitems++] = ((unsigned)il.pass_t[k][lane] << 4) | (unsigned)p;   // (partner slot, sph_id-1)
      }
    }
    if (!slow) slow = !push_boundary(post0, post1, o, B, c, L, nitems);
  }
  return slow ? 0 : nitems;
}

}  // namespace
}  // namespace af3d
