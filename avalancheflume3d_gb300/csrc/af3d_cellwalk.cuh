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

// The same index from the FP32 culling coordinate xf and the FP32 grid copies: the estimate
// q = (xf - xmin) * inv is within 2^-24 ((|x| + |xmin|) inv + 3 q) (1 + 2^-20) of the exact
// quotient (four roundings), so when it is farther than eight times that bound from every
// integer it truncates to the reference's index; otherwise (and for q near 0 or below) the FP64
// path decides.
__device__ __forceinline__ long search_axis_f(float xf, float xminf, float invf, double x, double xmin, double side,
                                              double inv, long n) {
  const float q = (xf - xminf) * invf;
  const float E = 4.76837158203125e-07f * ((fabsf(xf) + fabsf(xminf)) * invf + 3.0f * q);   // 2^-21 (...)
  if (q > E && q < 4.0e6f) {
    const float tq = truncf(q);
    const float fr = q - tq;   // exact: q and tq lie within a factor two of each other
    if (fr > E && fr < 1.0f - E) {
      long i = (long)tq;
      if (i == n) i--;
      return i;
    }
  }
  return search_axis(x, xmin, side, inv, n);
}

__device__ __forceinline__ Search search_centre_f(float4 cf, V3 r, const af3d_cell_par &g, const GridF &gf,
                                                  long long off) {
  Search q;
  q.off = off;
  q.ci = search_axis_f(cf.x, gf.xmin, gf.ix, r.x, g.rr_min.x, g.cell_side.x, g.cs_inv.x, g.ncell.x);
  q.cj = search_axis_f(cf.y, gf.ymin, gf.iy, r.y, g.rr_min.y, g.cell_side.y, g.cs_inv.y, g.ncell.y);
  q.ck = search_axis_f(cf.z, gf.zmin, gf.iz, r.z, g.rr_min.z, g.cell_side.z, g.cs_inv.z, g.ncell.z);
  return q;
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

constexpr int kLaneItems = kListCap;
constexpr unsigned kBndItem = 0xFFFFFF00u;   // boundary item: kBndItem | routine << 2 | sphere

// Partners per clump that pass the centre test; a clump with more takes the per-clump walk.  The
// benchmark states have at most 10 (262,144-clump bed, 524,288-clump polydisperse funnel); the
// cap sets most of the list phase's shared memory, which the L1 cache shares.
constexpr int kPassCap = 24;
constexpr unsigned kSlotMask = 0x3FFFFFFFu;   // pass entry: position or slot | (x offset + 1) << 30

// Per-warp partner lists of the two-stage gather in shared memory, one column per lane
// ([entry][lane]): a lane's own accesses always fall in its own bank.
struct PassLists {
  unsigned pass_t[kPassCap][32];         // partner position, then slot | (cell x offset + 1) << 30
  unsigned short pass_m[kPassCap][32];   // their 16-bit sphere-pair masks
  int pbase[33];
  unsigned short cand[kLaneItems][32];   // candidate sphere pairs in item order: entry << 4 | sph_id-1
                                         // (0x8000: rejected by the overlap test)
  int cbase[33];
};
static_assert(((kPassCap - 1) << 4 | 15) < 0x8000, "candidate entries are 15-bit");

// Item lists held in shared memory (the adjoint's cooperative reverse).
struct ItemLists {
  unsigned items[kLaneItems][32];
  int base[33];                          // exclusive prefix of the lanes' item counts
  PassLists pl;
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

// Boundary items of the routines [r0, r1] for one clump (culling record me), appended to the
// lane's item column `col` (entries `stride` apart); false if the list would overflow.  The FP32
// gates admit every sphere the routine can touch (and a few more, which the exact test of the
// force pass then rejects).
__device__ __forceinline__ bool push_boundary(int r0, int r1, const CullRec &me, const Consts &c, bool door_closed,
                                              unsigned *col, long stride, int &nitems) {
  for (int rt = r0; rt <= r1; rt++) {
    if (!bnd_may_touch_f(rt, me.c, me.c.w, c, door_closed)) continue;
    for (int ns = 0; ns < 4; ns++) {
      if (!bnd_may_touch_f(rt, me.s[ns], me.s[ns].w, c, door_closed)) continue;   // one sphere
      if (nitems == kLaneItems) return false;
      col[stride * nitems++] = kBndItem | (unsigned)(rt << 2) | (unsigned)ns;
    }
  }
  return true;
}

// Stage 1 of the gather (per lane): the partners among the 27 neighbour cells whose bounding
// spheres can touch the clump's (FP32 centre test), the clump itself included.  The three cells of one (jdel, kdel) row are
// consecutive in the linear cell index, so their members form one slot range split by four
// start[] values; the nine ranges are walked one after another, two slots a turn with both
// loads issued together.  Each kept partner is tagged with its cell's x offset (0..2) so that
// the reference's visiting order (idel, then jdel, kdel, then slot) can be restored.  Returns
// the number of partners found (which may exceed kPassCap).
__device__ __forceinline__ int gather_partners(PassLists &pl, long s, float4 mc, const Search &q,
                                               const af3d_cell_par &g, const int *__restrict__ start,
                                               const int *__restrict__ order, const float4 *__restrict__ csort,
                                               const CullRec *__restrict__ cull) {
  const int lane = threadIdx.x & 31;
  int npass = 0;
  // Kept partners are recorded by their position k in the (cell, id) order; stage 2 looks up
  // their slots (and drops the clump itself) with all lanes busy.
  auto keep = [&](int k, unsigned tag, float4 pc) {
    const float lim = mc.w + pc.w;
    if (d2f(mc, pc) > lim * lim * kCullSlack) return;
    if (npass < kPassCap) pl.pass_t[npass][lane] = (unsigned)k | (tag << 30);
    npass++;
  };
  const long x0 = q.ci - 1;
#pragma unroll 1
  for (int r = 0; r < 9; r++) {
    const long jn = q.cj + (r / 3 - 1), kn = q.ck + (r % 3 - 1);
    if (jn < 0 || kn < 0 || jn >= g.ncell.y || kn >= g.ncell.z) continue;
    const long rb = q.off + g.ncell.x * (jn + g.ncell.y * kn);
    // boundary e of the row: start of cell x0 + e, clamped into the row (empty cells outside)
    int b[4];
#pragma unroll
    for (int e = 0; e < 4; e++) {
      long x = x0 + e;
      x = x < 0 ? 0 : (x > g.ncell.x ? g.ncell.x : x);
      b[e] = __ldg(&start[rb + x]);
    }
    int k = b[0];
#pragma unroll 1
    for (; k + 1 < b[3]; k += 2) {
      const float4 p0 = order ? __ldg(&csort[k]) : cull[k].c;
      const float4 p1 = order ? __ldg(&csort[k + 1]) : cull[k + 1].c;
      keep(k, 1u + (k >= b[1]) + (k >= b[2]), p0);
      keep(k + 1, 1u + (k + 1 >= b[1]) + (k + 1 >= b[2]), p1);
    }
    if (k < b[3]) keep(k, 1u + (k >= b[1]) + (k >= b[2]), order ? __ldg(&csort[k]) : cull[k].c);
  }
  return npass;
}

// Every lane's item list of one contact pass, in the reference's order: the boundary routines
// before the particles (avalanche: hop x3, funnel, fcorners, walls), the particle contacts
// sph_id-major, the routines after them (avalanche: flume; fill: hop x3).  Boundary items
// (routine, sphere) for the spheres the routine's 1-Lipschitz gate cannot rule out; particle
// items (partner slot, sph_id) from a three-stage gather: stage 1 (per lane, gather_partners)
// keeps the partners whose bounding spheres can touch, stage 2 (whole warp) runs the sixteen
// FP32 sphere tests of every kept partner, 32 a round, and stage 3 (whole warp) the exact FP64
// overlap test of every sphere pair the FP32 test could not rule out.  Items go to the lane's column `col`, entries
// `stride` apart.  All 32 lanes call this; returns the lane's item count, 0 with `slow` set
// when the lane's lists would overflow.
// (the counts of a clump's list: `pre` boundary items, then `pair` particle items, then the rest)
struct ListCounts {
  int pre, pair;
};

__device__ __forceinline__ int build_item_lists(PassLists &pl, unsigned *col, long stride, long wbase, long s,
                                                bool act, bool aval, V3 r, const Consts &c,
                                                const af3d_cell_par &g, const GridF &gf, long long off,
                                                const NbrRec *__restrict__ nbr,
                                                const CullRec *__restrict__ cull, const int *__restrict__ start,
                                                const int *__restrict__ order, const float4 *__restrict__ csort,
                                                bool &slow, ListCounts &lc) {
  const int lane = threadIdx.x & 31;
  const int pre0 = aval ? R_HOP0 : 1, pre1 = aval ? R_WALLS : 0;         // fill: none before
  const int post0 = aval ? R_FLUME : R_HOP0, post1 = aval ? R_FLUME : R_HOP2;
  int nitems = 0;
  slow = false;
  lc.pre = lc.pair = 0;
  const CullRec me = cull[s];
  const bool door_closed = *c.tp < 0.0;
  if (act) slow = !push_boundary(pre0, pre1, me, c, door_closed, col, stride, nitems);
  lc.pre = nitems;
  int npass = 0;
  if (act && !slow) {
    npass = gather_partners(pl, s, me.c, search_centre_f(me.c, r, g, gf, off), g, start, order, csort, cull);
    if (npass > kPassCap) {
      slow = true;
      npass = 0;
    }
  }
  // Stage 2 (whole warp): each kept partner's slot, then its sixteen sphere tests, 32 partners a
  // round (the clump itself gets an empty mask).
  const int total_pass = warp_prefix(npass, pl.pbase);
  for (int j0 = 0; j0 < total_pass; j0 += 32) {
    const int j = j0 + lane;
    if (j < total_pass) {
      const int ow = owner_of(pl.pbase, j), k = j - pl.pbase[ow];
      const unsigned e = pl.pass_t[k][ow];
      const int pos = (int)(e & kSlotMask);
      const int t = order ? __ldg(&order[pos]) : pos;
      pl.pass_t[k][ow] = (unsigned)t | (e & ~kSlotMask);
      pl.pass_m[k][ow] = t == wbase + ow ? (unsigned short)0 : (unsigned short)sphere_mask(cull[wbase + ow], cull[t]);
    }
  }
  __syncwarp();
  // Each lane's candidate sphere pairs in item order: sph_id-major (the order of the sixteen
  // force_part launches), and within one sph_id in the reference's cell order (x offset, then
  // row, then slot).  Partners without a candidate sphere pair are dropped first (keeping the
  // walk order), and only the sph_ids some partner has are visited.
  int ncand = 0;
  if (act && !slow) {
    int m = 0;
    unsigned any = 0u;
#pragma unroll 1
    for (int k = 0; k < npass; k++) {
      const unsigned mk16 = pl.pass_m[k][lane];
      if (!mk16) continue;
      pl.pass_t[m][lane] = pl.pass_t[k][lane];
      pl.pass_m[m][lane] = (unsigned short)mk16;
      any |= mk16;
      m++;
    }
#pragma unroll 1
    while (any && !slow) {
      const int p = __ffs(any) - 1;
      any &= any - 1u;
#pragma unroll 1
      for (unsigned tag = 1; tag <= 3 && !slow; tag++)
#pragma unroll 1
        for (int k = 0; k < m; k++) {
          if ((pl.pass_t[k][lane] >> 30) != tag || !((pl.pass_m[k][lane] >> p) & 1u)) continue;
          if (nitems + ncand == kLaneItems) {
            slow = true;
            break;
          }
          pl.cand[ncand++][lane] = (unsigned short)(((unsigned)k << 4) | (unsigned)p);
        }
    }
    if (slow) ncand = 0;
  }
  // Stage 3 (whole warp): the exact FP64 overlap test of every candidate (the test the force
  // pass would make first), 32 a round, so that the force pass gets only overlapping pairs.
  const int total_cand = warp_prefix(ncand, pl.cbase);
  for (int j0 = 0; j0 < total_cand; j0 += 32) {
    const int j = j0 + lane;
    if (j < total_cand) {
      const int ow = owner_of(pl.cbase, j), ci = j - pl.cbase[ow];
      const unsigned e = pl.cand[ci][ow];
      const int k = (int)(e >> 4), p = (int)(e & 15u);
      const NbrRec &mo = nbr[wbase + ow];
      const V3 s1 = mk(mo.s[3 * (p & 3)], mo.s[3 * (p & 3) + 1], mo.s[3 * (p & 3) + 2]);
      V3 d;
      double dist2, sep;
      if (!spheres_overlap(s1, mo.rad, nbr[pl.pass_t[k][ow] & kSlotMask], p >> 2, d, dist2, sep))
        pl.cand[ci][ow] = (unsigned short)(e | 0x8000u);
    }
  }
  __syncwarp();
  if (act && !slow) {
#pragma unroll 1
    for (int i = 0; i < ncand; i++) {
      const unsigned e = pl.cand[i][lane];
      if (e & 0x8000u) continue;
      const unsigned t = pl.pass_t[e >> 4][lane] & kSlotMask;
      col[stride * nitems++] = (t << 4) | (e & 15u);   // (partner slot, sph_id-1)
    }
    lc.pair = nitems - lc.pre;
    slow = !push_boundary(post0, post1, me, c, door_closed, col, stride, nitems);
  }
  return slow ? 0 : nitems;
}

}  // namespace
}  // namespace af3d
