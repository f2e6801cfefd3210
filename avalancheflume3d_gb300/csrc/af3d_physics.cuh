// af3d_physics.cuh -- per-clump FP64 physics of the reference step, as device functions.
//
// Exact mode (the default build): every expression keeps the reference's FP64 evaluation order,
// and the translation units that include this header are compiled with -fmad=false, so a force,
// torque or acceleration computed here is bit-identical to the reference host routine on the
// same input (+, -, *, / and sqrt are correctly rounded on both sides).  Only init_Verlet's
// sin/cos come from CUDA's libm, which may differ from the host libm in the last bit.
//
// Fast mode (built with -DAF3D_FAST -fmad=true): the same FP64 physics with multiply-adds
// contracted, normals and tangents from a reciprocal square root instead of three divisions,
// and quotients by a shared divisor taken as products with one reciprocal.  Each of these
// changes a result by a few units in the last place, so forces agree with the reference to
// ~1e-14 relative rather than bit for bit.
//
// Geometry stays exact in both modes.  The distances that decide whether a contact exists, and
// whose difference from the radius is the contact's compression, are evaluated with
// non-contracting intrinsics (__dmul_rn, __dadd_rn, __dsub_rn: never fused into a multiply-add)
// in the reference's order, and the centre distance of a sphere pair or a funnel corner is the
// correctly rounded sqrt: the squared distance of two sphere centres, the slope-frame
// coordinates, the distance to the flume bed and to the funnel walls.  A compression is a
// difference of nearly equal numbers: the plane distances cancel coordinates of up to ~100 cm,
// a sphere-pair distance cancels against the radii, down to compressions of 1e-7 cm or less in
// a freshly loaded contact, so a different last bit (~1e-14 cm for a plane, ~3e-17 cm for a
// pair) would change such a contact's force by up to ~1e-7 (plane) or ~1e-9 (pair) of itself.
// Kept exact, the fast mode takes every overlap decision and computes every compression as the
// exact mode does.
#pragma once

#include "af3d_internal.h"

namespace af3d {

#ifdef AF3D_FAST
constexpr bool kFast = true;
#else
constexpr bool kFast = false;
#endif

// cabecera.hu:5-19
constexpr double kPI = 3.1415926535897932;
constexpr double kGRAV = 981.0;
constexpr double kGYR = 4.4494897427831781;
constexpr double kSPH_FACT = 4.188790204786391;
constexpr double kROOT2 = 1.414213562373095;
constexpr double kDRAG = 1.895e-3;
constexpr double kHOP_HEIGHT = 25.0;
constexpr double kHOP_WIDTH = 15.0;
constexpr double kYFUNNEL = 30.0;
constexpr double kLFUNNEL = 70.0;
constexpr double kYHOP_L = 7.5;
constexpr double kYHOP_R = 22.5;

struct V3 {
  double x, y, z;
};

__device__ __forceinline__ V3 mk(double x, double y, double z) {
  V3 r;
  r.x = x; r.y = y; r.z = z;
  return r;
}

// ---- FP64 tests and conversions on the integer pipe ----------------------------------------
// The FP64 pipe of this GPU retires one warp instruction per ~19 SM cycles, and conversions and
// comparisons of doubles occupy it like arithmetic does.  These helpers take the same decisions
// and give the same bits as the hardware instructions they replace, from the operands' bit
// patterns, on the integer pipe; values outside their fast range (zero, subnormal or huge
// results, infinities, NaN) fall back to the hardware conversion.

// isfinite(x): the exponent field is not all ones.
__device__ __forceinline__ bool finite_bits(double x) {
  return ((unsigned)(__double_as_longlong(x) >> 32) & 0x7FF00000u) != 0x7FF00000u;
}

// x != 0.0 (true for NaN, false for both zeros).
__device__ __forceinline__ bool nonzero_bits(double x) {
  return (__double_as_longlong(x) << 1) != 0;
}

// lo < x < hi for 0 <= lo < hi finite and x >= +0 or NaN (false for NaN, as the FP compare).
__device__ __forceinline__ bool in_open_range_bits(double x, double lo, double hi) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned long long l = (unsigned long long)__double_as_longlong(lo);
  return b - l - 1ull < (unsigned long long)__double_as_longlong(hi) - l - 1ull;
}

// (float)x, round to nearest even: the top 23 mantissa bits, rounded on the 29 below.
__device__ __forceinline__ float to_float_rn(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const int e = (int)((hi >> 20) & 0x7FFu) - 896;   // the float's biased exponent
  if (e <= 0 || e >= 255) return (float)x;
  const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29), rest = lo & 0x1FFFFFFFu;
  unsigned f = (hi & 0x80000000u) | ((unsigned)e << 23) | m;
  f += (rest > 0x10000000u) | ((rest == 0x10000000u) & (m & 1u));   // a carry into the exponent is right
  return __uint_as_float(f);
}

// __double2float_ru(x), rounded toward +infinity.
__device__ __forceinline__ float to_float_ru(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
  const int e = (int)((hi >> 20) & 0x7FFu) - 896;
  if (e <= 0 || e >= 255) return __double2float_ru(x);
  const unsigned m = ((hi & 0xFFFFFu) << 3) | (lo >> 29), rest = lo & 0x1FFFFFFFu;
  unsigned f = (hi & 0x80000000u) | ((unsigned)e << 23) | m;
  f += (rest != 0u) & !(hi >> 31);   // away from zero for positive x, toward zero for negative
  return __uint_as_float(f);
}

// (long long)x, truncated toward zero.
__device__ __forceinline__ long long trunc_to_ll(double x) {
  const long long b = __double_as_longlong(x);
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  if (e < 0) return 0;                      // |x| < 1, zeros and subnormals included
  if (e > 51) return (long long)x;          // integral already, or not finite
  const unsigned long long m = ((unsigned long long)b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
  const long long i = (long long)(m >> (52 - e));
  return b < 0 ? -i : i;
}

// The constants of flume f, loaded per thread (contexts with several flumes).
__device__ __forceinline__ Consts load_consts(const DevScalars *d, int f) {
  const DevFlume &fl = d->flumes[f];
  return make_consts(fl.sys, fl.fun, fl.tant, d->phase, d->variant, &d->time);
}

// time > 0 && x > side.x (init_Verlet.cu:29, cells.cu:65, force_part.cu:47, ...)
__device__ __forceinline__ bool is_removed(double time, double x, double side_x) {
  return time > 0.0 && x > side_x;
}

// Spring-dashpot normal force + Cundall-Strack tangential force with the Coulomb cap; the common
// tail of every contact type (force_part.cu:189-241, force_walls.cu:123-177, ...).
//   xi0:  Coulomb branch also when xi was zeroed (walls; DEV particle variant)
//   gate: false -> proceed when normal > 0; true -> proceed unless normal <= 0 (fcorners)
__device__ __forceinline__ bool contact_law_fast(V3 dvvc, V3 n, double comp, double km, double gm,
                                                 double mass_t, double mu, double cns_1, double dt,
                                                 double inv_dt, bool xi0, bool gate, V3 &f) {
  const double vn = dvvc.x * n.x + dvvc.y * n.y + dvvc.z * n.z;
  const V3 vt = mk(dvvc.x - vn * n.x, dvvc.y - vn * n.y, dvvc.z - vn * n.z);
  const double vt2 = vt.x * vt.x + vt.y * vt.y + vt.z * vt.z;
  const double inv_vt = rsqrt(vt2);          // +inf for vt = 0: the tangential part is then NaN
  const double vt_mag = vt2 * inv_vt;        // and skipped, as in the exact law
  // dvvc . vt / |vt| = |vt| up to the rounding of vt's orthogonality to n, which the exact law
  // also rounds: the fast law takes |vt| itself
  const double vt_sig = vt_mag;
  const double normal = km * comp + gm * (-vn);
  if (gate ? (normal <= 0.0) : !(normal > 0.0)) return false;
  f = mk(-normal * n.x, -normal * n.y, -normal * n.z);
  double xi = dt * vt_sig;
  if (cns_1 * normal < fabs(xi)) xi = 0.0;
  const double fsdt = 1.0e12 * mass_t * xi + 2.0e6 * mass_t * (xi * inv_dt);
  if (vt_mag > 0.0) {
    if (fabs(fsdt) > mu * normal || (xi0 && xi == 0.0)) {
      // af = 0.8 mu N / |vt|, t0 = m / af, af / (1 + (dt / t0)^2) = af m^2 / (m^2 + (dt af)^2)
      const double af = 0.8 * mu * normal * inv_vt;
      const double dta = dt * af;
      const double a = af * (mass_t * mass_t) / (mass_t * mass_t + dta * dta);
      f.x += a * vt.x;
      f.y += a * vt.y;
      f.z += a * vt.z;
    } else {
      const double q = fsdt * inv_vt;
      if (nonzero_bits(vt.x)) f.x += q * vt.x;
      if (nonzero_bits(vt.y)) f.y += q * vt.y;
      if (nonzero_bits(vt.z)) f.z += q * vt.z;
    }
  }
  return true;
}

__device__ __forceinline__ bool contact_law(V3 dvvc, V3 n, double comp, double km, double gm,
                                            double mass_t, double mu, double cns_1, double dt,
                                            bool xi0, bool gate, V3 &f) {
  double vn = dvvc.x * n.x + dvvc.y * n.y + dvvc.z * n.z;
  V3 vt;
  vt.x = dvvc.x - vn * n.x;
  vt.y = dvvc.y - vn * n.y;
  vt.z = dvvc.z - vn * n.z;
  double vt_mag = sqrt(vt.x * vt.x + vt.y * vt.y + vt.z * vt.z);
  V3 tv;
  tv.x = vt.x / vt_mag;
  tv.y = vt.y / vt_mag;
  tv.z = vt.z / vt_mag;
  double vt_sig = dvvc.x * tv.x + dvvc.y * tv.y + dvvc.z * tv.z;
  double normal = km * comp + gm * (-vn);
  if (gate ? (normal <= 0.0) : !(normal > 0.0)) return false;
  f.x = -normal * n.x;
  f.y = -normal * n.y;
  f.z = -normal * n.z;
  double xi = dt * vt_sig;
  if (cns_1 * normal < fabs(xi)) xi = 0.0;
  double xi_dot = xi / dt;
  double fsdt = 1.0e12 * mass_t * xi + 2.0e6 * mass_t * xi_dot;
  if (vt_mag > 0.0) {
    // Coulomb branch:  af = 0.8 mu N / |vt|; t0 = m / af; af /= 1 + (dt/t0)^2; f += af vt.
    // Otherwise:       f_i += fsdt vt_i / |vt| where vt_i != 0.
    // The two branches' first three divisions run as one sequence with per-lane operands, so
    // a warp whose lanes take different branches executes three divisions, not seven; every
    // lane still evaluates exactly its own branch's operations.
    const bool coulomb = fabs(fsdt) > mu * normal || (xi0 && xi == 0.0);
    const double q1 = (coulomb ? 0.8 * mu * normal : fsdt * vt.x) / vt_mag;   // af  | f_x term
    const double q2 = (coulomb ? mass_t : fsdt * vt.y) / (coulomb ? q1 : vt_mag);   // t0 | f_y
    const double q3 = (coulomb ? dt : fsdt * vt.z) / (coulomb ? q2 : vt_mag);   // dt/t0 | f_z
    if (coulomb) {
      const double af = q1 / (1.0 + q3 * q3);
      f.x += af * vt.x;
      f.y += af * vt.y;
      f.z += af * vt.z;
    } else {
      if (nonzero_bits(vt.x)) f.x += q1;
      if (nonzero_bits(vt.y)) f.y += q2;
      if (nonzero_bits(vt.z)) f.z += q3;
    }
  }
  return true;
}

// v + w x (c - r) in the reference's operand order (force_part.cu:175-177).
__device__ __forceinline__ V3 point_velocity(V3 v, V3 w, V3 c, V3 r) {
  V3 u;
  u.x = v.x + w.y * (c.z - r.z) - w.z * (c.y - r.y);
  u.y = v.y + w.z * (c.x - r.x) - w.x * (c.z - r.z);
  u.z = v.z + w.x * (c.y - r.y) - w.y * (c.x - r.x);
  return u;
}

// The own clump as the force routines see it.
struct Own {
  V3 r, v, w;
  V3 s[4];
  double rad, mwall, msph;
};

// One sphere of a clump as a boundary routine sees it: clump centre, velocities, sphere
// centre, radius and the wall-contact mass.
struct Sph {
  V3 r, v, w, s;
  double rad, mwall;
};

__device__ __forceinline__ Sph sphere_of(const Own &o, int ns) {
  Sph q;
  q.r = o.r; q.v = o.v; q.w = o.w; q.s = o.s[ns]; q.rad = o.rad; q.mwall = o.mwall;
  return q;
}

// The terms T += (c - r) x fs adds (force_part.cu:245-251), one component each.
__device__ __forceinline__ V3 torque_term(V3 c, V3 r, V3 fs) {
  return mk((c.y - r.y) * fs.z - (c.z - r.z) * fs.y, (c.z - r.z) * fs.x - (c.x - r.x) * fs.z,
            (c.x - r.x) * fs.y - (c.y - r.y) * fs.x);
}

// T += tq; F += fs (force_part.cu:245-251 with tq = torque_term(c, r, fs)).
__device__ __forceinline__ void add_terms(V3 &F, V3 &T, V3 fs, V3 tq) {
  T.x += tq.x; T.y += tq.y; T.z += tq.z;
  F.x += fs.x; F.y += fs.y; F.z += fs.z;
}

// Everything the contact law needs about one contact, from either a sphere pair or a sphere and
// a wall: the relative velocity at the contact point, the normal, the compression, the spring
// and dashpot coefficients, the tangential mass, friction and its cap, and the law's switches.
struct ContactIn {
  V3 dvvc, n, rrc;
  double comp, km, gm, mass_t, mu, cns;
  bool xi0, gate;
};

// Wall contact of one sphere at contact point rrc with outward normal n (force_walls.cu:106-177
// and the same tail in every boundary routine).
__device__ __forceinline__ void wall_input(const Sph &o, V3 rrc, V3 n, double comp, const Consts &c,
                                           bool gate, ContactIn &ci) {
  if (kFast) {   // the same law with the constant halves formed once per flume
    ci.km = c.hk_pw * o.mwall;
    ci.gm = c.hg_pw * o.mwall;
  } else {
    ci.km = 0.5 * c.kappa_pw * o.mwall;
    ci.gm = 0.5 * c.gamma_pw * o.mwall;
  }
  V3 vvc = point_velocity(o.v, o.w, rrc, o.r);
  ci.dvvc = mk(-vvc.x, -vvc.y, -vvc.z);
  ci.n = n;
  ci.rrc = rrc;
  ci.comp = comp;
  ci.mass_t = o.mwall;
  ci.mu = c.mu_pw;
  ci.cns = c.cns_pw;
  ci.xi0 = true;
  ci.gate = gate;
}

// The contact law on a prepared contact: force fs and its torque term about the clump centre r.
__device__ __forceinline__ bool apply_law(const ContactIn &ci, V3 r, const Consts &c, V3 &fs, V3 &tq) {
  const bool on = kFast ? contact_law_fast(ci.dvvc, ci.n, ci.comp, ci.km, ci.gm, ci.mass_t, ci.mu, ci.cns, c.dt,
                                           c.inv_dt, ci.xi0, ci.gate, fs)
                        : contact_law(ci.dvvc, ci.n, ci.comp, ci.km, ci.gm, ci.mass_t, ci.mu, ci.cns, c.dt,
                                      ci.xi0, ci.gate, fs);
  if (!on) return false;
  tq = torque_term(ci.rrc, r, fs);
  return true;
}

// rotate_vectors.cu:28-30 (lab -> slope frame; uncontracted in both modes) and
// force_funnel.cu:88-93 (slope -> lab).
__device__ __forceinline__ V3 to_slope(V3 r, double cost, double sint) {
  return mk(__dsub_rn(__dmul_rn(r.x, cost), __dmul_rn(r.z, sint)), r.y,
            __dadd_rn(__dmul_rn(r.x, sint), __dmul_rn(r.z, cost)));
}
__device__ __forceinline__ V3 to_lab(V3 q, double cost, double sint) {
  return mk(q.x * cost + q.z * sint, q.y, q.z * cost - q.x * sint);
}

// The per-sphere bodies of the boundary routines: the force of routine `routine` on one sphere
// (false: no force).  Each routine adds its spheres' terms in sphere order a, b, c, d.

// force_hop.cu:9-244, wall group nw, one sphere.
__device__ __forceinline__ bool hop_sphere(const Sph &o, int nw, const Consts &c, ContactIn &ci) {
  const double ri = o.rad;
  const V3 s = o.s;
  V3 rrc, n;
  double dist, comp = 0.0;
  int touch = 0;
  if (s.z < kHOP_HEIGHT || s.x > kHOP_WIDTH) return false;
  if (nw == 0) {
    dist = s.x - 0.0;
    if (dist <= ri) { touch = 1; rrc = mk(0.0, s.y, s.z); n = mk(-1.0, 0.0, 0.0); comp = ri - dist; }
    dist = kHOP_WIDTH - s.x;
    if (dist <= ri) { touch = 2; rrc = mk(kHOP_WIDTH, s.y, s.z); n = mk(1.0, 0.0, 0.0); comp = ri - dist; }
  } else if (nw == 1) {
    dist = s.y - kYHOP_L;
    if (dist <= ri) { touch = 3; rrc = mk(s.x, kYHOP_L, s.z); n = mk(0.0, -1.0, 0.0); comp = ri - dist; }
    dist = kYHOP_R - s.y;
    if (dist <= ri) { touch = 4; rrc = mk(s.x, kYHOP_R, s.z); n = mk(0.0, 1.0, 0.0); comp = ri - dist; }
  } else {
    dist = s.z - kHOP_HEIGHT;
    if (dist <= ri) {
      touch = *c.tp < 0.0 ? 5 : 0;   // the door is open once time >= 0 (force_hop.cu:140-143)
      rrc = mk(s.x, s.y, kHOP_HEIGHT); n = mk(0.0, 0.0, -1.0); comp = ri - dist;
    }
  }
  if (!touch) return false;
  wall_input(o, rrc, n, comp, c, false, ci);
  return true;
}

// force_funnel.cu:9-213, one sphere.
__device__ __forceinline__ bool funnel_sphere(const Sph &o, const Consts &c, ContactIn &ci) {
  const double ri = o.rad;
  V3 q = to_slope(o.s, c.cost, c.sint), qc, nr, rrc, n;
  double dist, comp = 0.0;
  int touch = 0;
  if (q.x > __dsub_rn(kLFUNNEL, __dmul_rn(ri, c.sinfi))) return false;
  dist = fabs(__dsub_rn(q.y, __dmul_rn(q.x, c.tanfi))) * c.cosfi;
  if (dist <= ri) {
    touch = 1;
    qc = mk(q.x + dist * c.sinfi, q.y - dist * c.cosfi, q.z);
    nr = mk(c.sinfi, -c.cosfi, 0.0);
    rrc = to_lab(qc, c.cost, c.sint);
    n = to_lab(nr, c.cost, c.sint);
    comp = ri - dist;
  }
  dist = fabs(__dsub_rn(kYFUNNEL - q.y, __dmul_rn(q.x, c.tanfi))) * c.cosfi;
  if (dist <= ri) {
    touch = 2;
    qc = mk(q.x + dist * c.sinfi, q.y + dist * c.cosfi, q.z);
    nr = mk(c.sinfi, c.cosfi, 0.0);
    rrc = to_lab(qc, c.cost, c.sint);
    n = to_lab(nr, c.cost, c.sint);
    comp = ri - dist;
  }
  if (!touch) return false;
  wall_input(o, rrc, n, comp, c, false, ci);
  return true;
}

// force_funnel.cu:216-404, one sphere.
__device__ __forceinline__ bool fcorners_sphere(const Sph &o, const Consts &c, ContactIn &ci) {
  const double ri = o.rad;
  const double yfun_l = c.dy2, yfun_r = c.side_y + c.dy2, hsy = c.dy2 + c.side_y / 2.0;
  V3 q = to_slope(o.s, c.cost, c.sint);
  if (q.x < __dsub_rn(kLFUNNEL, __dmul_rn(ri, c.sinfi)) || q.x > kLFUNNEL + ri) return false;
  if (q.y > yfun_r || q.y < yfun_l) return false;
  double yc = (q.y <= hsy) ? yfun_l : yfun_r;
  double sep2 = ri * ri;
  V3 d;
  d.x = kLFUNNEL - q.x;
  double dist2 = d.x * d.x;
  if (dist2 > sep2) return false;
  d.y = yc - q.y;
  dist2 = __dadd_rn(dist2, __dmul_rn(d.y, d.y));
  if (dist2 > sep2) return false;
  double dist;
  V3 nr;
  if (kFast) {
    const double inv = rsqrt(dist2);
    dist = sqrt(dist2);   // correctly rounded: the compression ri - dist is the exact mode's
    nr = mk(d.x * inv, d.y * inv, 0.0);
  } else {
    dist = sqrt(dist2);
    nr = mk(d.x / dist, d.y / dist, 0.0);
  }
  V3 qc = mk(q.x + ri * nr.x, q.y + ri * nr.y, q.z);
  wall_input(o, to_lab(qc, c.cost, c.sint), to_lab(nr, c.cost, c.sint), ri - dist, c, true, ci);
  return true;
}

// force_walls.cu:9-199, one sphere (callers skip removed clumps).
__device__ __forceinline__ bool walls_sphere(const Sph &o, const Consts &c, ContactIn &ci) {
  const double ri = o.rad;
  const double yleft = c.dy2, yright = c.side_y + c.dy2;
  const V3 s = o.s;
  V3 rrc, n;
  if (to_slope(s, c.cost, c.sint).x <= kLFUNNEL) return false;
  double dist, comp = 0.0;
  int touch = 0;
  dist = s.y - yleft;
  if (dist <= ri) { touch = 1; rrc = mk(s.x, yleft, s.z); n = mk(0.0, -1.0, 0.0); comp = ri - dist; }
  dist = yright - s.y;
  if (dist <= ri) { touch = 2; rrc = mk(s.x, yright, s.z); n = mk(0.0, 1.0, 0.0); comp = ri - dist; }
  if (!touch) return false;
  wall_input(o, rrc, n, comp, c, false, ci);
  return true;
}

// force_flume.cu:10-182, one sphere (callers skip removed clumps).
__device__ __forceinline__ bool flume_sphere(const Sph &o, const Consts &c, ContactIn &ci) {
  const double ri = o.rad;
  const double tant = c.tant;   // c.sint / c.cost, formed once per flume by the host
  const V3 s = o.s;
  double rect = __dsub_rn(__dmul_rn(-tant, s.x), s.z);
  double dist = fabs(c.cost * rect);
  if (!(dist <= ri)) return false;
  const V3 n = mk(-c.sint, 0.0, -c.cost);
  V3 rrc = mk(s.x - dist * c.sint, s.y, s.z - dist * c.cost);
  wall_input(o, rrc, n, ri - dist, c, false, ci);
  return true;
}

// The contact of routine `routine` with one sphere, prepared for the law (false: no contact).
__device__ __forceinline__ bool bnd_input(int routine, const Sph &o, const Consts &c, ContactIn &ci) {
  switch (routine) {
    case R_HOP0: return hop_sphere(o, 0, c, ci);
    case R_HOP1: return hop_sphere(o, 1, c, ci);
    case R_HOP2: return hop_sphere(o, 2, c, ci);
    case R_FUNNEL: return funnel_sphere(o, c, ci);
    case R_FCORNERS: return fcorners_sphere(o, c, ci);
    case R_WALLS: return walls_sphere(o, c, ci);
    case R_FLUME: return flume_sphere(o, c, ci);
  }
  return false;
}

// The force of routine `routine` on one sphere and its torque term (false: no force).
__device__ __forceinline__ bool bnd_sphere(int routine, const Sph &o, const Consts &c, V3 &fs, V3 &tq) {
  ContactIn ci;
  return bnd_input(routine, o, c, ci) && apply_law(ci, o.r, c, fs, tq);
}

// One boundary routine over the four spheres of a clump, with the reference's removed-clump
// rule for that routine (walls and flume skip removed clumps; hop, funnel, fcorners do not).
__device__ __forceinline__ void bnd_routine(int routine, const Own &o, bool removed, const Consts &c,
                                            V3 &F, V3 &T) {
  if (removed && (routine == R_WALLS || routine == R_FLUME)) return;
#pragma unroll 1
  for (int ns = 0; ns < 4; ns++) {
    V3 fs, tq;
    if (bnd_sphere(routine, sphere_of(o, ns), c, fs, tq)) add_terms(F, T, fs, tq);
  }
}

// Whether a boundary routine can touch any sphere of a clump whose spheres lie within distance
// B of its centre r (B >= max sphere offset + radius, rounded up).  Every distance a boundary
// routine tests is a 1-Lipschitz function of the sphere centre (plane distances, coordinates in
// the rotated frame), so if the centre's value misses the routine's threshold by more than B no
// sphere can pass the test and the routine adds nothing.  The margin `eps` covers the FP64
// rounding of these centre expressions.  Used to skip routines, never to change their result.
__device__ __forceinline__ bool bnd_may_touch(int routine, V3 r, double B, const Consts &c) {
  const double eps = 1e-12 * (1.0 + fabs(r.x) + fabs(r.y) + fabs(r.z));
  const double Bm = B + eps;
  switch (routine) {
    case R_HOP0: case R_HOP1: case R_HOP2: {
      if (r.z + Bm < kHOP_HEIGHT || r.x - Bm > kHOP_WIDTH) return false;   // force_hop.cu:67
      if (routine == R_HOP0) return r.x <= Bm || r.x >= kHOP_WIDTH - Bm;
      if (routine == R_HOP1) return r.y - kYHOP_L <= Bm || kYHOP_R - r.y <= Bm;
      return *c.tp < 0.0 && r.z - kHOP_HEIGHT <= Bm;
    }
    case R_FUNNEL: {
      const double xr = r.x * c.cost - r.z * c.sint, yr = r.y;
      if (xr - Bm > kLFUNNEL) return false;
      return fabs(yr - xr * c.tanfi) * c.cosfi <= Bm || fabs(kYFUNNEL - yr - xr * c.tanfi) * c.cosfi <= Bm;
    }
    case R_FCORNERS: {
      const double xr = r.x * c.cost - r.z * c.sint;
      return fabs(xr - kLFUNNEL) <= 2.0 * Bm;
    }
    case R_WALLS: {
      const double xr = r.x * c.cost - r.z * c.sint;
      if (xr + Bm <= kLFUNNEL) return false;
      return r.y - c.dy2 <= Bm || c.side_y + c.dy2 - r.y <= Bm;
    }
    case R_FLUME: {
      const double zr = r.x * c.sint + r.z * c.cost;
      return fabs(zr) <= Bm;
    }
  }
  return true;
}

// bnd_may_touch in FP32 on the culling record's coordinates p (each the FP32 rounding of the
// FP64 value) and bound B (rounded up).  Each routine's expression is at most five FP32
// operations on values below ~10^3 and constants rounded to FP32, so it lies within
// ~10 * 2^-24 (|x| + |y| + |z| + 30) of the exact value; the slack S below is more than twice
// that (and covers the FP64 rounding of the routine's own test), so every position the FP64
// gate (and hence the routine) can pass also passes here.  door_closed: time < 0.
__device__ __forceinline__ bool bnd_may_touch_f(int routine, float4 p, float B, const Consts &c, bool door_closed) {
  const float S = 1e-5f * (101.0f + fabsf(p.x) + fabsf(p.y) + fabsf(p.z));
  const float Bm = B + S;
  switch (routine) {
    case R_HOP0: case R_HOP1: case R_HOP2: {
      if (p.z + Bm < (float)kHOP_HEIGHT || p.x - Bm > (float)kHOP_WIDTH) return false;
      if (routine == R_HOP0) return p.x <= Bm || p.x >= (float)kHOP_WIDTH - Bm;
      if (routine == R_HOP1) return p.y - (float)kYHOP_L <= Bm || (float)kYHOP_R - p.y <= Bm;
      return door_closed && p.z - (float)kHOP_HEIGHT <= Bm;
    }
    case R_FUNNEL: {
      const float xr = p.x * c.cost_f - p.z * c.sint_f, yr = p.y;
      if (xr - Bm > (float)kLFUNNEL) return false;
      return fabsf(yr - xr * c.tanfi_f) * c.cosfi_f <= Bm ||
             fabsf((float)kYFUNNEL - yr - xr * c.tanfi_f) * c.cosfi_f <= Bm;
    }
    case R_FCORNERS: {
      const float xr = p.x * c.cost_f - p.z * c.sint_f;
      return fabsf(xr - (float)kLFUNNEL) <= 2.0f * Bm;
    }
    case R_WALLS: {
      const float xr = p.x * c.cost_f - p.z * c.sint_f;
      if (xr + Bm <= (float)kLFUNNEL) return false;
      return p.y - c.dy2_f <= Bm || c.side_y_f + c.dy2_f - p.y <= Bm;
    }
    case R_FLUME: {
      const float zr = p.x * c.sint_f + p.z * c.cost_f;
      return fabsf(zr) <= Bm;
    }
  }
  return true;
}

// One sphere-sphere contact of force_part.cu:139-241: own sphere s1 (clump centre rrl), partner
// record m, partner sphere sm.  Returns false when the staged test finds no overlap; otherwise
// the contact is prepared for the law.
// The staged overlap test of force_part.cu:143-157 between own sphere s1 (radius rad_1) and
// sphere sm of partner m: d = s2 - s1, dist2 = |d|^2 and sep = rad_1 + rad_2.  The reference
// compares each partial sum of dist2 with sep^2; the partial sums never decrease (each adds a
// square and rounding is monotone, fused or not), so the last comparison alone takes the same
// decision, NaN included.  The list kernel and pair_input run this same function.
__device__ __forceinline__ bool spheres_overlap(const V3 &s1, double rad_1, const NbrRec &m, int sm, V3 &d,
                                                double &dist2, double &sep, bool known = false) {
  const double rad_2 = m.rad;
  sep = rad_1 + rad_2;
  const double sep2 = sep * sep;
  d.x = m.s[3 * sm] - s1.x;
  d.y = m.s[3 * sm + 1] - s1.y;
  d.z = m.s[3 * sm + 2] - s1.z;
  dist2 = d.x * d.x;
  dist2 = __dadd_rn(dist2, __dmul_rn(d.y, d.y));   // uncontracted in both modes
  dist2 = __dadd_rn(dist2, __dmul_rn(d.z, d.z));
  return known || dist2 < sep2;   // known: an item of the lists, which this same test kept
}

// listed: the pair is an item of the lists, whose overlap test (this one) it passed.
__device__ __forceinline__ bool pair_input(const V3 &rrl, const V3 &vvl, const V3 &wwl, const V3 &s1,
                                           double rad_1, double massl, const NbrRec &m, int sm,
                                           const Consts &c, bool xi0, ContactIn &ci, bool listed = false) {
  V3 d;
  double dist2, sep;
  if (!spheres_overlap(s1, rad_1, m, sm, d, dist2, sep, listed)) return false;
  if (kFast) {   // 0.5 kappa 0.5 (m1 + m2) with kappa / 4 formed once per flume
    const double msum = m.msph + massl;
    ci.km = c.qk_pp * msum;
    ci.gm = c.qg_pp * msum;
  } else {
    const double meff = 0.5 * (m.msph + massl);
    ci.km = 0.5 * c.kappa_pp * meff;
    ci.gm = 0.5 * c.gamma_pp * meff;
  }
  double dist;
  if (kFast) {
    const double inv = rsqrt(dist2);
    dist = sqrt(dist2);   // correctly rounded: the compression sep - dist is the exact mode's
    ci.n = mk(d.x * inv, d.y * inv, d.z * inv);
  } else {
    dist = sqrt(dist2);
    ci.n = mk(d.x / dist, d.y / dist, d.z / dist);
  }
  ci.rrc = mk(s1.x + rad_1 * ci.n.x, s1.y + rad_1 * ci.n.y, s1.z + rad_1 * ci.n.z);
  V3 vl = point_velocity(vvl, wwl, ci.rrc, rrl);
  V3 vm = point_velocity(mk(m.vx, m.vy, m.vz), mk(m.wx, m.wy, m.wz), ci.rrc, mk(m.rx, m.ry, m.rz));
  ci.dvvc = mk(vm.x - vl.x, vm.y - vl.y, vm.z - vl.z);
  ci.comp = sep - dist;
  ci.mass_t = massl;
  ci.mu = c.mu_pp;
  ci.cns = c.cns_pp;
  ci.xi0 = xi0;
  ci.gate = false;
  return true;
}

// The whole sphere-sphere contact: 0 (no overlap), 1 (overlap, no force) or 2 (force); with 2,
// fs is the contact force and tq its torque about rrl, the terms force_part.cu:245-251 adds.
__device__ __forceinline__ int part_pair_contrib(const V3 &rrl, const V3 &vvl, const V3 &wwl,
                                                 const V3 &s1, double rad_1, double massl,
                                                 const NbrRec &m, int sm, const Consts &c, bool xi0,
                                                 V3 &fs, V3 &tq) {
  ContactIn ci;
  if (!pair_input(rrl, vvl, wwl, s1, rad_1, massl, m, sm, c, xi0, ci)) return 0;
  return apply_law(ci, rrl, c, fs, tq) ? 2 : 1;
}

// The same contact accumulated into (F, T) in place.
__device__ __forceinline__ int part_pair(const V3 &rrl, const V3 &vvl, const V3 &wwl, const V3 &s1,
                                         double rad_1, double massl, const NbrRec &m, int sm,
                                         const Consts &c, bool xi0, V3 &F, V3 &T) {
  V3 fs, tq;
  const int r = part_pair_contrib(rrl, vvl, wwl, s1, rad_1, massl, m, sm, c, xi0, fs, tq);
  if (r == 2) {
    T.x += tq.x; T.y += tq.y; T.z += tq.z;
    F.x += fs.x; F.y += fs.y; F.z += fs.z;
  }
  return r;
}

// (+0 * a) * b as IEEE arithmetic evaluates it for finite a and b: a zero whose sign is the
// exclusive-or of the signs of a and b.
__device__ __forceinline__ double signed_zero_product(double a, double b) {
  const unsigned long long sa = (unsigned long long)__double_as_longlong(a);
  const unsigned long long sb = (unsigned long long)__double_as_longlong(b);
  return __longlong_as_double((long long)((sa ^ sb) & 0x8000000000000000ull));
}

// get_accel.cu:21-75 for one clump; R rows Rx, Ry, Rz.  `adrag0` = DRAG*rad*rad/m (the same
// expression, precomputed per clump).  For isotropic inertia (Ix == Iy == Iz, the reference's
// clumps, calculate_particle_parameters.cu:33) the Euler coupling terms C*wb*wb are (+0*wb)*wb,
// i.e. signed zeros; they are formed from the sign bits instead of two divisions-by-I and four
// multiplications, which gives the same bits for finite angular velocities.
// (fast mode: im = 1/m and iI = 1/I.x, formed once at import, replace the divisions)
__device__ __forceinline__ void get_accel_one(V3 f, V3 t, V3 v, V3 w, V3 Rx, V3 Ry, V3 Rz, double m,
                                              double adrag0, V3 I, V3 &a, V3 &al, double im, double iI) {
  const double v2 = v.x * v.x + v.y * v.y + v.z * v.z;
  // fast mode: |v| from the reciprocal square root (the drag term is ~1e-3 of gravity here)
  double vmag = kFast ? (v2 == 0.0 ? 0.0 : v2 * rsqrt(v2)) : sqrt(v2);   // NaN stays NaN
  double adrag = adrag0 * vmag;
  if (kFast) {
    a.x = f.x * im - adrag * v.x;
    a.y = f.y * im - adrag * v.y;
    a.z = f.z * im - adrag * v.z - kGRAV;
  } else {
    a.x = f.x / m - adrag * v.x;
    a.y = f.y / m - adrag * v.y;
    a.z = f.z / m - adrag * v.z - kGRAV;
  }
  V3 wb, tb, ab;
  if (kFast && I.x == I.y && I.y == I.z && I.x > 0.0 && isfinite(I.x) && isfinite(w.x) && isfinite(w.y) &&
      isfinite(w.z)) {
    // Fast mode, isotropic inertia: the Euler term C w_b x w_b is zero (C = 0), so the body-frame
    // spin is not formed; alpha = R (R^T T) / I.
    tb.x = t.x * Rx.x + t.y * Ry.x + t.z * Rz.x;
    tb.y = t.x * Rx.y + t.y * Ry.y + t.z * Rz.y;
    tb.z = t.x * Rx.z + t.y * Ry.z + t.z * Rz.z;
    ab = mk(tb.x * iI, tb.y * iI, tb.z * iI);
    al.x = ab.x * Rx.x + ab.y * Rx.y + ab.z * Rx.z;
    al.y = ab.x * Ry.x + ab.y * Ry.y + ab.z * Ry.z;
    al.z = ab.x * Rz.x + ab.y * Rz.y + ab.z * Rz.z;
    return;
  }
  wb.x = w.x * Rx.x + w.y * Ry.x + w.z * Rz.x;
  wb.y = w.x * Rx.y + w.y * Ry.y + w.z * Rz.y;
  wb.z = w.x * Rx.z + w.y * Ry.z + w.z * Rz.z;
  tb.x = t.x * Rx.x + t.y * Ry.x + t.z * Rz.x;
  tb.y = t.x * Rx.y + t.y * Ry.y + t.z * Rz.y;
  tb.z = t.x * Rx.z + t.y * Ry.z + t.z * Rz.z;
  if (I.x == I.y && I.y == I.z && isfinite(wb.x) && isfinite(wb.y) && isfinite(wb.z) && I.x > 0.0 &&
      isfinite(I.x)) {
    if (kFast) {
      ab.x = tb.x * iI + signed_zero_product(wb.y, wb.z);
      ab.y = tb.y * iI + signed_zero_product(wb.z, wb.x);
      ab.z = tb.z * iI + signed_zero_product(wb.x, wb.y);
    } else {
      ab.x = tb.x / I.x + signed_zero_product(wb.y, wb.z);
      ab.y = tb.y / I.y + signed_zero_product(wb.z, wb.x);
      ab.z = tb.z / I.z + signed_zero_product(wb.x, wb.y);
    }
  } else {
    double Cxy = (I.x - I.y) / I.z;
    double Cyz = (I.y - I.z) / I.x;
    double Czx = (I.z - I.x) / I.y;
    ab.x = tb.x / I.x + Cyz * wb.y * wb.z;
    ab.y = tb.y / I.y + Czx * wb.z * wb.x;
    ab.z = tb.z / I.z + Cxy * wb.x * wb.y;
  }
  al.x = ab.x * Rx.x + ab.y * Rx.y + ab.z * Rx.z;
  al.y = ab.x * Ry.x + ab.y * Ry.y + ab.z * Ry.z;
  al.z = ab.x * Rz.x + ab.y * Rz.y + ab.z * Rz.z;
}

// DRAG*rad*rad/m in get_accel.cu:47's operand order.
__device__ __forceinline__ double drag_factor(double rad, double m) { return kDRAG * rad * rad / m; }

}  // namespace af3d
