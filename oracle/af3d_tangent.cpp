/*
 * af3d_tangent.cpp -- FP64 CPU tangent-linear model of the clump-DEM step.
 *
 * TEST INFRASTRUCTURE ONLY: the forward-mode reference that the engine's adjoint
 * (af3d_adjoint) is checked against.  The product path never links, loads or calls it.
 *
 * It is af3d_oracle.c compiled a second time, as C++, with the oracle's real type set to a
 * dual number: every value carries kDirs directional derivatives, propagated through each
 * +, -, *, / and sqrt, sin, cos, fabs by the chain rule.  Values are formed by the same
 * operations in the same order as in the oracle (built with -ffp-contract=off as well), so
 * the value trajectory is bit-identical to the oracle's, and every discrete decision
 * (cells, contact sets, Coulomb or elastic branch, removal) follows the values: the
 * derivatives are those of the same piecewise-smooth path the adjoint differentiates.
 *
 * At a point where a derivative does not exist, a one-sided choice is made: d sqrt(x) = 0 at
 * x = 0 (the drag term's |v| at rest, where the product with v vanishes anyway) and
 * d|x| = dx at x = 0.
 *
 * Entry point (C ABI): tlm_run -- the start-up force pass and `steps` steps of the phase from
 * a state with tangents on the system parameters and on the particle state, returning
 * J = sum m (x cos(tilt) - z sin(tilt)) / sum m over all clumps at the end and its directional
 * derivatives.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

namespace af3d_tlm {

constexpr int kDirs = 8;   // directions carried per run

struct Dual {
  double v;
  double d[kDirs];
  Dual() = default;
  Dual(double x) : v(x) {
    for (int k = 0; k < kDirs; k++) d[k] = 0.0;
  }
  explicit operator long() const { return (long)v; }
  explicit operator int() const { return (int)v; }
};

inline Dual operator+(const Dual &a, const Dual &b) {
  Dual r;
  r.v = a.v + b.v;
  for (int k = 0; k < kDirs; k++) r.d[k] = a.d[k] + b.d[k];
  return r;
}
inline Dual operator-(const Dual &a, const Dual &b) {
  Dual r;
  r.v = a.v - b.v;
  for (int k = 0; k < kDirs; k++) r.d[k] = a.d[k] - b.d[k];
  return r;
}
inline Dual operator-(const Dual &a) {
  Dual r;
  r.v = -a.v;
  for (int k = 0; k < kDirs; k++) r.d[k] = -a.d[k];
  return r;
}
inline Dual operator+(const Dual &a) { return a; }
inline Dual operator*(const Dual &a, const Dual &b) {
  Dual r;
  r.v = a.v * b.v;
  for (int k = 0; k < kDirs; k++) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
  return r;
}
inline Dual operator/(const Dual &a, const Dual &b) {
  Dual r;
  r.v = a.v / b.v;
  for (int k = 0; k < kDirs; k++) r.d[k] = (a.d[k] - r.v * b.d[k]) / b.v;
  return r;
}
inline Dual &operator+=(Dual &a, const Dual &b) { return a = a + b; }
inline Dual &operator-=(Dual &a, const Dual &b) { return a = a - b; }
inline Dual &operator*=(Dual &a, const Dual &b) { return a = a * b; }
inline Dual &operator/=(Dual &a, const Dual &b) { return a = a / b; }

inline bool operator<(const Dual &a, const Dual &b) { return a.v < b.v; }
inline bool operator<=(const Dual &a, const Dual &b) { return a.v <= b.v; }
inline bool operator>(const Dual &a, const Dual &b) { return a.v > b.v; }
inline bool operator>=(const Dual &a, const Dual &b) { return a.v >= b.v; }
inline bool operator==(const Dual &a, const Dual &b) { return a.v == b.v; }
inline bool operator!=(const Dual &a, const Dual &b) { return a.v != b.v; }

inline Dual sqrt(const Dual &a) {
  Dual r;
  r.v = ::sqrt(a.v);
  const double s = r.v > 0.0 ? 0.5 / r.v : 0.0;
  for (int k = 0; k < kDirs; k++) r.d[k] = a.d[k] * s;
  return r;
}
inline Dual sin(const Dual &a) {
  Dual r;
  r.v = ::sin(a.v);
  const double c = ::cos(a.v);
  for (int k = 0; k < kDirs; k++) r.d[k] = a.d[k] * c;
  return r;
}
inline Dual cos(const Dual &a) {
  Dual r;
  r.v = ::cos(a.v);
  const double s = -::sin(a.v);
  for (int k = 0; k < kDirs; k++) r.d[k] = a.d[k] * s;
  return r;
}
inline Dual fabs(const Dual &a) { return a.v < 0.0 ? -a : a; }

}  // namespace af3d_tlm

#define ORC_REAL af3d_tlm::Dual
#include "af3d_oracle.c"

namespace {

using af3d_tlm::Dual;
using af3d_tlm::kDirs;

// The oracle's structs hold `nlong` integers followed by `nreal` reals, in the same order in
// the double layout (the reference's) and in the dual layout.
static_assert(sizeof(orc_particle) == 51 * sizeof(Dual), "particle layout");
static_assert(sizeof(orc_system_par) == sizeof(long) + 31 * sizeof(Dual), "system_par layout");
static_assert(sizeof(orc_funnel) == 3 * sizeof(Dual), "funnel layout");
static_assert(sizeof(orc_cell_par) == 6 * sizeof(long) + 15 * sizeof(Dual), "cell_par layout");

// One struct from the double layout, with direction k's tangent of real j read from
// tan[k * tan_stride + j] (tan null: no tangents).
template <class S>
void lift(S &out, const unsigned char *in, int nlong, int nreal, const double *tan, long tan_stride, int ndir) {
  unsigned char *o = reinterpret_cast<unsigned char *>(&out);
  memcpy(o, in, sizeof(long) * nlong);
  const double *x = reinterpret_cast<const double *>(in + sizeof(long) * nlong);
  Dual *y = reinterpret_cast<Dual *>(o + sizeof(long) * nlong);
  for (int j = 0; j < nreal; j++) {
    y[j] = Dual(x[j]);
    for (int k = 0; k < ndir && tan; k++) y[j].d[k] = tan[k * tan_stride + j];
  }
}

// Values of a dual-layout struct back into the double layout.
template <class S>
void drop(unsigned char *out, const S &in, int nlong, int nreal) {
  const unsigned char *i = reinterpret_cast<const unsigned char *>(&in);
  memcpy(out, i, sizeof(long) * nlong);
  const Dual *x = reinterpret_cast<const Dual *>(i + sizeof(long) * nlong);
  double *y = reinterpret_cast<double *>(out + sizeof(long) * nlong);
  for (int j = 0; j < nreal; j++) y[j] = x[j].v;
}

}  // namespace

extern "C" __attribute__((visibility("default"))) int tlm_directions(void) { return kDirs; }

/* Host threads of the per-clump loops (the oracle's own OpenMP loops over clumps, each
   writing only its own clump's entries, so the result does not depend on the count). */
extern "C" __attribute__((visibility("default"))) void tlm_set_threads(int nthreads) {
  orc_set_threads(nthreads);
}

/* The start-up force pass (orc_forces, then a_i = a_f) and `steps` orc_step calls of the phase
   and friction variant, from the state (sys, fun, cell, pp[n]) in the reference's layouts, with
   accelerations zero at the start.  ndir <= tlm_directions() directions: dsys[k] (a system_par,
   double layout; npart ignored) and dpp[k * n + i] (a particle) hold direction k's tangents of
   the system parameters and of clump i's state; either may be null (no tangent).  Writes J and
   dJ[k] for k < ndir, and (pp_out non-null) the final state's values.  Returns an ORC_* status
   (or -1 for a bad argument). */
extern "C" __attribute__((visibility("default"))) int tlm_run(const void *sys, const void *fun, const void *cell,
                                                             const void *pp, long n, int ndir, const double *dsys,
                                                             const double *dpp, long steps, int phase, int variant,
                                                             double *J, double *dJ, void *pp_out) {
  if (ndir < 0 || ndir > kDirs || n < 0 || steps < 0 || !sys || !fun || !cell || (n > 0 && !pp) || !J)
    return -1;
  orc_system_par s;
  orc_funnel f;
  orc_cell_par c;
  lift(s, static_cast<const unsigned char *>(sys), 1, 31, dsys ? dsys + 1 : nullptr, 32, ndir);
  lift(f, static_cast<const unsigned char *>(fun), 0, 3, nullptr, 0, 0);
  lift(c, static_cast<const unsigned char *>(cell), 6, 15, nullptr, 0, 0);
  std::vector<orc_particle> p((size_t)n);
  for (long i = 0; i < n; i++)
    lift(p[i], static_cast<const unsigned char *>(pp) + 408 * i, 0, 51, dpp ? dpp + 51 * i : nullptr, 51 * n, ndir);
  std::vector<orc_vec3> buf((size_t)6 * (n > 0 ? n : 1), orc_vec3{Dual(0.0), Dual(0.0), Dual(0.0)});
  std::vector<long> cell_vec((size_t)(c.ntot > 0 ? c.ntot : 1), -1);
  std::vector<int> nocup((size_t)(c.ncell3 > 0 ? c.ncell3 : 1), 0);
  const long m = n > 0 ? n : 1;
  orc_work w;
  w.force = buf.data();
  w.torque = buf.data() + m;
  w.acc_i = buf.data() + 2 * m;
  w.anga_i = buf.data() + 3 * m;
  w.acc_f = buf.data() + 4 * m;
  w.anga_f = buf.data() + 5 * m;
  w.cell_vec = cell_vec.data();
  w.nocup_vec = nocup.data();
  w.cell_vec_cap = (long)cell_vec.size();
  w.nocup_cap = (long)nocup.size();
  int st = orc_forces(&s, &f, &c, p.data(), &w, phase, variant);
  if (st != ORC_OK) return st;
  orc_vec3 *t = w.acc_i;
  w.acc_i = w.acc_f;
  w.acc_f = t;
  t = w.anga_i;
  w.anga_i = w.anga_f;
  w.anga_f = t;
  for (long k = 0; k < steps; k++) {
    st = orc_step(&s, &f, &c, p.data(), &w, phase, variant);
    if (st != ORC_OK) return st;
  }
  Dual mx(0.0), mt(0.0);
  for (long i = 0; i < n; i++) {
    mx += p[i].mass * (p[i].rr.x * s.cost - p[i].rr.z * s.sint);
    mt += p[i].mass;
  }
  const Dual q = mt.v > 0.0 ? mx / mt : Dual(0.0);
  *J = q.v;
  for (int k = 0; k < ndir && dJ; k++) dJ[k] = q.d[k];
  if (pp_out)
    for (long i = 0; i < n; i++) drop(static_cast<unsigned char *>(pp_out) + 408 * i, p[i], 0, 51);
  return ORC_OK;
}
