// af3d_adjoint.cu -- reverse-mode derivative (adjoint) of the exact-mode step.
//
// The forward step, with its discrete structure held fixed (cells, contact sets, which branch of
// the contact law and which wall each sphere touches):
//   predict    r1 = r + dt (v + dt/2 a_i),  v1 = v + dt a_i,  w1 = w + dt alpha_i,
//              R1 = colnorm(dR(dO) R) with dO = dt (w + dt/2 alpha_i),  s_k = r1 + pos R1 p_k
//   forces     F, T = sum over contacts and walls (each a function of the two clumps' r1, v1,
//              w1 and sphere centres, and of kappa, gamma, mu)
//   get_accel  a_f = F/m - drag |v1| v1 - g z,  alpha_f = R1 (R1^T T) / I
//   finish     v2 = v1 + dt/2 (a_f - a_i),  w2 = w1 + dt/2 (alpha_f - alpha_i)
// and the next state is (r1, v2, w2, R1, a_f, alpha_f).  The kernels here run that step
// backwards: given the adjoint of the next state they form the adjoint of this one, and add the
// step's contributions to the adjoints of kappa, gamma and mu (particle and wall).  Every
// contact is re-evaluated from the step's recomputed state; the derivative of the contact law
// is its exact piecewise derivative, including the Coulomb-capped sliding branch.  A contact's
// derivative with respect to the partner clump is scattered with FP64 atomics: derivatives of a
// sum do not depend on the order of its terms.
//
// Compiled with -fmad=false like the exact step kernels (the forward re-evaluation must take
// the forward's branches).
#include "af3d_adjoint.cuh"
#include "af3d_cellwalk.cuh"

namespace af3d {

namespace {

// Adjoints of the law's inputs.
struct LawBar {
  V3 dv, n;
  double comp, km, gm, mu;
};

// The contact law (contact_law, af3d_physics.cuh, exact mode) and its reverse in one pass.  The
// forward part repeats contact_law's operations in its order (same branches, same force f); it
// returns false when the contact produced no force.  Then, with the adjoints fb_tot, tb_tot of
// the owner's force and torque sums and the lever e (torque += e x f), it forms the adjoints of
// the law's inputs (lb) and adds that of the lever to e_b.  The derivative needs no bit-exact
// quotient: one reciprocal of |vt| serves all of it.
__device__ __forceinline__ bool contact_law_fwd_rev(const ContactIn &ci, double dt, V3 fb_tot, V3 tb_tot, V3 e,
                                                    V3 &e_b, LawBar &lb) {
  // forward, as contact_law
  const V3 dv = ci.dvvc, n = ci.n;
  const double vn = dv.x * n.x + dv.y * n.y + dv.z * n.z;
  V3 vt;
  vt.x = dv.x - vn * n.x;
  vt.y = dv.y - vn * n.y;
  vt.z = dv.z - vn * n.z;
  const double vt_mag = sqrt(vt.x * vt.x + vt.y * vt.y + vt.z * vt.z);
  V3 tv;
  tv.x = vt.x / vt_mag;
  tv.y = vt.y / vt_mag;
  tv.z = vt.z / vt_mag;
  const double vt_sig = dv.x * tv.x + dv.y * tv.y + dv.z * tv.z;
  const double normal = ci.km * ci.comp + ci.gm * (-vn);
  if (ci.gate ? (normal <= 0.0) : !(normal > 0.0)) return false;
  V3 f;
  f.x = -normal * n.x;
  f.y = -normal * n.y;
  f.z = -normal * n.z;
  double xi = dt * vt_sig;
  const bool zeroed = ci.cns * normal < fabs(xi);
  if (zeroed) xi = 0.0;
  const double xi_dot = xi / dt;
  const double m = ci.mass_t;
  const double fsdt = 1.0e12 * m * xi + 2.0e6 * m * xi_dot;
  const bool tang = vt_mag > 0.0;
  const bool coul = tang && (fabs(fsdt) > ci.mu * normal || (ci.xi0 && xi == 0.0));
  double q1 = 0.0, q3 = 0.0;
  if (tang) {
    q1 = (coul ? 0.8 * ci.mu * normal : fsdt * vt.x) / vt_mag;
    const double q2 = (coul ? m : fsdt * vt.y) / (coul ? q1 : vt_mag);
    q3 = (coul ? dt : fsdt * vt.z) / (coul ? q2 : vt_mag);
    if (coul) {
      const double af = q1 / (1.0 + q3 * q3);
      f.x += af * vt.x;
      f.y += af * vt.y;
      f.z += af * vt.z;
    } else {
      if (vt.x != 0.0) f.x += q1;
      if (vt.y != 0.0) f.y += q2;
      if (vt.z != 0.0) f.z += q3;
    }
  }
  // reverse: F += f, T += e x f
  const V3 fb = fb_tot + cross(tb_tot, e);
  e_b += cross(f, tb_tot);
  double normal_b = -dot(fb, n);
  V3 n_b = (-normal) * fb;
  V3 dv_b = mk(0.0, 0.0, 0.0), vt_b = mk(0.0, 0.0, 0.0);
  double vtmag_b = 0.0, mu_b = 0.0;
  if (tang) {
    const double ivt = 1.0 / vt_mag;
    if (coul) {
      // af = 0.8 mu N / |vt| (q1);  r = dt / (m / af) (q3);  f += af / (1 + r^2) vt
      const double af = q1, r = q3;
      const double iden = 1.0 / (1.0 + r * r);
      const double af2 = af * iden;
      const double af2_b = dot(fb, vt);
      vt_b = madd(af2, fb, vt_b);
      const double af_b = af2_b * (1.0 - r * r) * (iden * iden);
      mu_b += af_b * 0.8 * normal * ivt;
      normal_b += af_b * 0.8 * ci.mu * ivt;
      vtmag_b -= af_b * af * ivt;
    } else {
      // f_i += fsdt vt_i / |vt| for every component with vt_i != 0
      const double g = fsdt * ivt;
      double g_b = 0.0;
      if (vt.x != 0.0) { vt_b.x += g * fb.x; g_b += fb.x * vt.x; }
      if (vt.y != 0.0) { vt_b.y += g * fb.y; g_b += fb.y * vt.y; }
      if (vt.z != 0.0) { vt_b.z += g * fb.z; g_b += fb.z * vt.z; }
      const double fsdt_b = g_b * ivt;
      vtmag_b -= g_b * g * ivt;
      if (!zeroed) {
        // fsdt = m xi (1e12 + 2e6 / dt), xi = dt vt_sig, vt_sig = dv . vt / |vt|
        const double xi_b = fsdt_b * (1.0e12 * m + 2.0e6 * m / dt);
        const double vtsig_b = dt * xi_b;
        dv_b = madd(vtsig_b, tv, dv_b);
        const V3 tv_b = vtsig_b * dv;
        vt_b = madd(ivt, tv_b, vt_b);
        vtmag_b -= dot(tv_b, vt) * (ivt * ivt);
      }
    }
    vt_b = madd(vtmag_b, tv, vt_b);   // |vt| = sqrt(vt . vt)
  }
  // normal = km comp - gm vn
  lb.km = normal_b * ci.comp;
  lb.comp = normal_b * ci.km;
  lb.gm = -normal_b * vn;
  double vn_b = -normal_b * ci.gm;
  // vt = dv - vn n
  dv_b += vt_b;
  vn_b -= dot(vt_b, n);
  n_b = madd(-vn, vt_b, n_b);
  // vn = dv . n
  dv_b = madd(vn_b, n, dv_b);
  n_b = madd(vn_b, dv, n_b);
  lb.dv = dv_b;
  lb.n = n_b;
  lb.mu = mu_b;
  return true;
}

// Adjoint accumulators of one clump's contact inputs.
struct ClumpBar {
  V3 r, v, w;
  V3 s[4];
};

// The owner's adjoints from one contact item: centre, velocities and the item's own sphere.
struct ItemBar {
  V3 r, v, w, s;
};

__device__ __forceinline__ ItemBar zero_item() {
  ItemBar b;
  b.r = b.v = b.w = b.s = mk(0.0, 0.0, 0.0);
  return b;
}

__device__ __forceinline__ void add_item(ClumpBar &ob, const ItemBar &ib, int k) {
  ob.r += ib.r;
  ob.v += ib.v;
  ob.w += ib.w;
  ob.s[k] += ib.s;
}

struct ParamBar {
  double kappa_pp, gamma_pp, mu_pp, kappa_pw, gamma_pw, mu_pw;
};

// Reverse of one sphere-sphere contact (pair_input + contact law + torque term) of the owner
// (centre rl, velocities vl, wl, sphere s1 = own sphere k) with partner record m, sphere sm.
// fb_tot / tb_tot: adjoints of the owner's force and torque sums.  Returns the partner's
// adjoints in pb (centre, velocities, sphere sm).
__device__ __forceinline__ void pair_rev(V3 rl, V3 vl, V3 wl, V3 s1, double rad1, double massl, const NbrRec &m,
                                         int sm, const Consts &c, bool xi0, V3 fb_tot, V3 tb_tot, ItemBar &ob,
                                         V3 &pr_b, V3 &pv_b, V3 &pw_b, V3 &ps_b, ParamBar &par, bool &any) {
  any = false;
  ContactIn ci;
  if (!pair_input(rl, vl, wl, s1, rad1, massl, m, sm, c, xi0, ci)) return;
  const V3 rrc = ci.rrc;
  const V3 e_l = rrc - rl;
  // F += f; T += e_l x f
  V3 e_l_b = mk(0.0, 0.0, 0.0);
  LawBar lb;
  if (!contact_law_fwd_rev(ci, c.dt, fb_tot, tb_tot, e_l, e_l_b, lb)) return;
  any = true;
  const V3 sp = mk(m.s[3 * sm], m.s[3 * sm + 1], m.s[3 * sm + 2]);
  const V3 rm = mk(m.rx, m.ry, m.rz), wm = mk(m.wx, m.wy, m.wz);
  const V3 d = sp - s1;
  const double dist = sqrt(d.x * d.x + d.y * d.y + d.z * d.z);
  const V3 n = ci.n;
  const V3 e_m = rrc - rm;
  const double meff = 0.5 * (m.msph + massl);
  par.kappa_pp += lb.km * 0.5 * meff;
  par.gamma_pp += lb.gm * 0.5 * meff;
  par.mu_pp += lb.mu;
  // dv = vm - vl;  vm = vm_lin + wm x e_m;  vl = vl_lin + wl x e_l
  const V3 vm_b = lb.dv, vl_b = (-1.0) * lb.dv;
  pv_b = vm_b;
  pw_b = cross(e_m, vm_b);
  V3 e_m_b = cross(vm_b, wm);
  ob.v += vl_b;
  ob.w += cross(e_l, vl_b);
  e_l_b += cross(vl_b, wl);
  // e_l = rrc - rl;  e_m = rrc - rm
  const V3 rrc_b = e_l_b + e_m_b;
  ob.r -= e_l_b;
  pr_b = (-1.0) * e_m_b;
  // rrc = s1 + rad1 n;  comp = sep - dist;  n = d / dist;  d = sp - s1
  V3 n_b = madd(rad1, rrc_b, lb.n);
  const double dist_b = -lb.comp;
  const V3 d_b = madd(dist_b, n, (1.0 / dist) * madd(-dot(n, n_b), n, n_b));
  ob.s += rrc_b;
  ob.s -= d_b;
  ps_b = d_b;
}

// Geometry of one wall contact as its routine forms it (the touch the routine keeps), and the
// map from the adjoints of (contact point, normal, compression) back to the sphere centre.
__device__ __forceinline__ bool wall_geom(int rt, const Sph &o, const Consts &c, V3 &rrc, V3 &n, double &comp,
                                          bool &gate, int &touch, double &aux) {
  const double ri = o.rad;
  const V3 s = o.s;
  touch = 0;
  gate = false;
  aux = 0.0;
  double dist;
  switch (rt) {
    case R_HOP0: case R_HOP1: case R_HOP2: {
      if (s.z < kHOP_HEIGHT || s.x > kHOP_WIDTH) return false;
      const int nw = rt - R_HOP0;
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
        if (dist <= ri && *c.tp < 0.0) {
          touch = 5; rrc = mk(s.x, s.y, kHOP_HEIGHT); n = mk(0.0, 0.0, -1.0); comp = ri - dist;
        }
      }
      return touch != 0;
    }
    case R_FUNNEL: {
      const V3 q = to_slope(s, c.cost, c.sint);
      if (q.x > kLFUNNEL - ri * c.sinfi) return false;
      double e = q.y - q.x * c.tanfi;
      dist = fabs(e) * c.cosfi;
      if (dist <= ri) {
        touch = 1; aux = e;
        rrc = to_lab(mk(q.x + dist * c.sinfi, q.y - dist * c.cosfi, q.z), c.cost, c.sint);
        n = to_lab(mk(c.sinfi, -c.cosfi, 0.0), c.cost, c.sint);
        comp = ri - dist;
      }
      e = kYFUNNEL - q.y - q.x * c.tanfi;
      dist = fabs(e) * c.cosfi;
      if (dist <= ri) {
        touch = 2; aux = e;
        rrc = to_lab(mk(q.x + dist * c.sinfi, q.y + dist * c.cosfi, q.z), c.cost, c.sint);
        n = to_lab(mk(c.sinfi, c.cosfi, 0.0), c.cost, c.sint);
        comp = ri - dist;
      }
      return touch != 0;
    }
    case R_FCORNERS: {
      const double yfun_l = c.dy2, yfun_r = c.side_y + c.dy2, hsy = c.dy2 + c.side_y / 2.0;
      const V3 q = to_slope(s, c.cost, c.sint);
      if (q.x < kLFUNNEL - ri * c.sinfi || q.x > kLFUNNEL + ri) return false;
      if (q.y > yfun_r || q.y < yfun_l) return false;
      const double yc = (q.y <= hsy) ? yfun_l : yfun_r;
      const double sep2 = ri * ri;
      V3 d;
      d.x = kLFUNNEL - q.x;
      double dist2 = d.x * d.x;
      if (dist2 > sep2) return false;
      d.y = yc - q.y;
      dist2 += d.y * d.y;
      if (dist2 > sep2) return false;
      dist = sqrt(dist2);
      const V3 nr = mk(d.x / dist, d.y / dist, 0.0);
      rrc = to_lab(mk(q.x + ri * nr.x, q.y + ri * nr.y, q.z), c.cost, c.sint);
      n = to_lab(nr, c.cost, c.sint);
      comp = ri - dist;
      gate = true;
      touch = 1;
      aux = yc;
      return true;
    }
    case R_WALLS: {
      const double yleft = c.dy2, yright = c.side_y + c.dy2;
      if (to_slope(s, c.cost, c.sint).x <= kLFUNNEL) return false;
      dist = s.y - yleft;
      if (dist <= ri) { touch = 1; rrc = mk(s.x, yleft, s.z); n = mk(0.0, -1.0, 0.0); comp = ri - dist; }
      dist = yright - s.y;
      if (dist <= ri) { touch = 2; rrc = mk(s.x, yright, s.z); n = mk(0.0, 1.0, 0.0); comp = ri - dist; }
      return touch != 0;
    }
    case R_FLUME: {
      const double rect = -c.tant * s.x - s.z;
      dist = fabs(c.cost * rect);
      if (!(dist <= ri)) return false;
      touch = 1;
      aux = c.cost * rect;
      rrc = mk(s.x - dist * c.sint, s.y, s.z - dist * c.cost);
      n = mk(-c.sint, 0.0, -c.cost);
      comp = ri - dist;
      return true;
    }
  }
  return false;
}

__device__ __forceinline__ double sgn(double x) { return x > 0.0 ? 1.0 : (x < 0.0 ? -1.0 : 0.0); }

// Sphere-centre adjoint from the adjoints of the wall contact's point, normal and compression.
__device__ __forceinline__ V3 wall_geom_rev(int rt, const Sph &o, const Consts &c, int touch, double aux, V3 rrc_b,
                                           V3 n_b, double comp_b) {
  const double ri = o.rad;
  switch (rt) {
    case R_HOP0: return mk(touch == 1 ? -comp_b : comp_b, rrc_b.y, rrc_b.z);
    case R_HOP1: return mk(rrc_b.x, touch == 3 ? -comp_b : comp_b, rrc_b.z);
    case R_HOP2: return mk(rrc_b.x, rrc_b.y, -comp_b);
    case R_WALLS: return mk(rrc_b.x, touch == 1 ? -comp_b : comp_b, rrc_b.z);
    case R_FUNNEL: {
      // q = S s; dist = |e| cosfi; qc = (q.x + dist sinfi, q.y -+ dist cosfi, q.z); rrc = L qc
      const V3 qc_b = to_slope(rrc_b, c.cost, c.sint);   // L^T = S
      const double side = touch == 1 ? -1.0 : 1.0;
      const double dist_b = -comp_b + qc_b.x * c.sinfi + side * qc_b.y * c.cosfi;
      const double ge = sgn(aux) * c.cosfi;   // d dist / d e
      // e = q.y - q.x tanfi (touch 1) or 30 - q.y - q.x tanfi (touch 2)
      const V3 q_b = mk(qc_b.x - dist_b * ge * c.tanfi, qc_b.y + (touch == 1 ? 1.0 : -1.0) * dist_b * ge, qc_b.z);
      return to_lab(q_b, c.cost, c.sint);   // S^T = L
    }
    case R_FCORNERS: {
      const V3 q = to_slope(o.s, c.cost, c.sint);
      const double dx = kLFUNNEL - q.x, dy = aux - q.y;
      const double dist = sqrt(dx * dx + dy * dy);
      const double nx = dx / dist, ny = dy / dist;
      const V3 qc_b = to_slope(rrc_b, c.cost, c.sint);
      const V3 nr_b3 = to_slope(n_b, c.cost, c.sint);
      const double nrx_b = nr_b3.x + ri * qc_b.x, nry_b = nr_b3.y + ri * qc_b.y;
      const double dist_b = -comp_b;
      const double proj = nx * nrx_b + ny * nry_b;
      const double ddx = (nrx_b - nx * proj) / dist + dist_b * nx;
      const double ddy = (nry_b - ny * proj) / dist + dist_b * ny;
      const V3 q_b = mk(qc_b.x - ddx, qc_b.y - ddy, qc_b.z);
      return to_lab(q_b, c.cost, c.sint);
    }
    case R_FLUME: {
      // rect = -tant s.x - s.z; dist = |cost rect|; rrc = (s.x - dist sint, s.y, s.z - dist cost)
      const double dist_b = -comp_b - rrc_b.x * c.sint - rrc_b.z * c.cost;
      const double g = sgn(aux) * c.cost;
      return mk(rrc_b.x - dist_b * g * c.tant, rrc_b.y, rrc_b.z - dist_b * g);
    }
  }
  return mk(0.0, 0.0, 0.0);
}

// Reverse of one wall contact of sphere k.
__device__ __forceinline__ void wall_rev(int rt, const Sph &o, const Consts &c, V3 fb_tot, V3 tb_tot, ItemBar &ob,
                                         ParamBar &par) {
  V3 rrc, n;
  double comp, aux;
  bool gate;
  int touch;
  if (!wall_geom(rt, o, c, rrc, n, comp, gate, touch, aux)) return;
  ContactIn ci;
  wall_input(o, rrc, n, comp, c, gate, ci);
  const V3 e = rrc - o.r;
  V3 e_b = mk(0.0, 0.0, 0.0);
  LawBar lb;
  if (!contact_law_fwd_rev(ci, c.dt, fb_tot, tb_tot, e, e_b, lb)) return;
  par.kappa_pw += lb.km * 0.5 * o.mwall;
  par.gamma_pw += lb.gm * 0.5 * o.mwall;
  par.mu_pw += lb.mu;
  // dv = -(v + w x e)
  const V3 vvc_b = (-1.0) * lb.dv;
  ob.v += vvc_b;
  ob.w += cross(e, vvc_b);
  e_b += cross(vvc_b, o.w);
  // e = rrc - r
  ob.r -= e_b;
  ob.s += wall_geom_rev(rt, o, c, touch, aux, e_b, lb.n, lb.comp);
}

__device__ __forceinline__ void warp_reduce_add(double *dst, double v) {
  for (int off = 16; off; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
  if ((threadIdx.x & 31) == 0 && v != 0.0) atomicAdd(dst, v);
}

// Adds every lane's value into dst[6 f + k] for the lane's flume f: one warp reduction when the
// warp's lanes share a flume, else one atomic per lane.  All 32 lanes call this.
__device__ __forceinline__ void add_params(double *dst, int f, const ParamBar &p) {
  const double v[6] = {p.kappa_pp, p.gamma_pp, p.mu_pp, p.kappa_pw, p.gamma_pw, p.mu_pw};
  const int f0 = __shfl_sync(0xffffffffu, f, 0);
  if (__all_sync(0xffffffffu, f == f0)) {
    for (int k = 0; k < 6; k++) warp_reduce_add(dst + 6 * f0 + k, v[k]);
  } else {
    for (int k = 0; k < 6; k++)
      if (v[k] != 0.0) atomicAdd(dst + 6 * f + k, v[k]);
  }
}

__device__ __forceinline__ void flush_params(double *dst, int f, const ParamBar &p) {
  const double v[6] = {p.kappa_pp, p.gamma_pp, p.mu_pp, p.kappa_pw, p.gamma_pw, p.mu_pw};
  for (int k = 0; k < 6; k++)
    if (v[k] != 0.0) atomicAdd(dst + 6 * f + k, v[k]);
}

// Every contact of one clump reversed by its own lane (the path of a clump whose item lists
// would overflow): walls of the phase, then every partner in the neighbour cells.
__device__ __forceinline__ void adj_contacts_lane(long s, const Own &o, const Consts &c, const af3d_cell_par &g,
                                                  long long off, double B, V3 Fb, V3 Tb, Planes acc,
                                                  const NbrRec *__restrict__ nbr, const CullRec *__restrict__ cull,
                                                  const int *__restrict__ start, const int *__restrict__ order,
                                                  ClumpBar &ob, ParamBar &par) {
  const bool aval = c.phase == AF3D_PHASE_AVALANCHE;
  for (int rt = R_HOP0; rt <= R_FLUME; rt++) {
    if (!aval && rt > R_HOP2) break;
    if (!bnd_may_touch(rt, o.r, B, c)) continue;
    for (int k = 0; k < 4; k++) {
      ItemBar ib = zero_item();
      wall_rev(rt, sphere_of(o, k), c, Fb, Tb, ib, par);
      add_item(ob, ib, k);
    }
  }
  const bool xi0 = c.variant == AF3D_FRICTION_DEV;
  const CullRec mine = cull[s];
  const Search q = search_centre(o.r, g, off);
  for_neighbour_slots(q, g, start, order, [&](int t) {
    if (t == s) return;
    unsigned mask = pair_mask(mine, cull[t]);
    while (mask) {
      const int p = __ffs(mask) - 1;
      mask &= mask - 1;
      const int k = p & 3, sm = p >> 2;
      V3 pr_b, pv_b, pw_b, ps_b;
      bool any;
      ItemBar ib = zero_item();
      pair_rev(o.r, o.v, o.w, o.s[k], o.rad, o.msph, nbr[t], sm, c, xi0, Fb, Tb, ib, pr_b, pv_b, pw_b, ps_b, par,
               any);
      add_item(ob, ib, k);
      if (any) {
        atomic_add3(acc, CR, t, pr_b);
        atomic_add3(acc, CV, t, pv_b);
        atomic_add3(acc, CW, t, pw_b);
        atomic_add3(acc, CS + 3 * sm, t, ps_b);
      }
    }
  });
}

constexpr int kAdjCoopBlock = 64;

// Per-warp shared state of the cooperative reverse: the item lists, every owner's force and
// torque adjoints, and every owner's contact adjoints (centre, v, w, four spheres) accumulated
// with shared-memory atomics (a reverse needs no order).
struct AdjQueue {
  ItemLists il;
  double fb[6][32];    // [component][lane]
  double own[21][32];  // [component][lane]
};

// Adds v to three components of one lane's column (component stride 32).
__device__ __forceinline__ void shared_add3(double *p, V3 v) {
  atomicAdd(p, v.x);
  atomicAdd(p + 32, v.y);
  atomicAdd(p + 64, v.z);
}

// Reverse of finish_Verlet and get_accel for clump s (startup: the start-up pass, which has no
// finish): out.a/out.al receive the finish terms of this step's a_i, alpha_i, rb the clump's own
// R1 adjoint; returns the adjoints of the force and torque sums (Fb, Tb) and of the predicted
// velocities (ob.v, ob.w).
__device__ __forceinline__ void adj_head(long s, bool act, bool valid, int startup, const Own &o, const Consts &c,
                                         const Planes &P, const Planes &in, const Planes &out, const Planes &rb,
                                         ClumpBar &ob, V3 &Fb, V3 &Tb) {
  ob.r = ob.v = ob.w = mk(0.0, 0.0, 0.0);
  for (int k = 0; k < 4; k++) ob.s[k] = mk(0.0, 0.0, 0.0);
  Fb = mk(0.0, 0.0, 0.0);
  Tb = mk(0.0, 0.0, 0.0);
  if (act) {
    // finish: v2 = v1 + hdt (a_f - a_i), w2 likewise
    const V3 v2_b = startup ? mk(0.0, 0.0, 0.0) : ld3(in, AV, s);
    const V3 w2_b = startup ? mk(0.0, 0.0, 0.0) : ld3(in, AW, s);
    const V3 af_b = ld3(in, AA, s) + c.hdt * v2_b;
    const V3 alf_b = ld3(in, AAL, s) + c.hdt * w2_b;
    if (!startup) {
      st3(out, AA, s, (-c.hdt) * v2_b);
      st3(out, AAL, s, (-c.hdt) * w2_b);
    }
    ob.v = v2_b;
    ob.w = w2_b;
    // get_accel: a_f = F/m - adrag0 |v1| v1 - g z;  alpha_f = R1 (R1^T T) / I (isotropic I)
    const double m = P.p[MASS][s], I = P.p[IXX][s], adrag0 = P.p[ADRAG][s];
    Fb = (1.0 / m) * af_b;
    const double vmag = sqrt(dot(o.v, o.v));
    if (vmag > 0.0) ob.v -= adrag0 * vmag * af_b + (adrag0 * dot(o.v, af_b) / vmag) * o.v;
    const V3 Rx = ld3(P, R00, s), Ry = ld3(P, R10, s), Rz = ld3(P, R20, s);
    const V3 T = ld3(P, TX, s);
    const V3 tb = mk(T.x * Rx.x + T.y * Ry.x + T.z * Rz.x, T.x * Rx.y + T.y * Ry.y + T.z * Rz.y,
                     T.x * Rx.z + T.y * Ry.z + T.z * Rz.z);
    const V3 ab = (1.0 / I) * tb;
    const V3 ab_b = mk(alf_b.x * Rx.x + alf_b.y * Ry.x + alf_b.z * Rz.x,
                       alf_b.x * Rx.y + alf_b.y * Ry.y + alf_b.z * Rz.y,
                       alf_b.x * Rx.z + alf_b.y * Ry.z + alf_b.z * Rz.z);
    const V3 tb_b = (1.0 / I) * ab_b;
    Tb = mk(dot(Rx, tb_b), dot(Ry, tb_b), dot(Rz, tb_b));
    // R1 adjoint: alpha_i = sum_j R_ij ab_j and tb_j = sum_i R_ij T_i
    V3 RbX = ld3(in, ARM, s), RbY = ld3(in, ARM + 3, s), RbZ = ld3(in, ARM + 6, s);
    RbX += alf_b.x * ab + T.x * tb_b;
    RbY += alf_b.y * ab + T.y * tb_b;
    RbZ += alf_b.z * ab + T.z * tb_b;
    st3(rb, 0, s, RbX);
    st3(rb, 3, s, RbY);
    st3(rb, 6, s, RbZ);
  } else if (valid) {
    for (int k = 0; k < 9; k++) rb.p[k][s] = 0.0;
    if (!startup) {
      st3(out, AA, s, mk(0.0, 0.0, 0.0));
      st3(out, AAL, s, mk(0.0, 0.0, 0.0));
    }
  }
}

// Reverse of one item of owner record om (force/torque adjoints fb_o, tb_o): the owner's adjoints
// in ib (returns the owner's sphere), the partner's straight into acc, the parameters' in ipar.
__device__ __forceinline__ int adj_item(const NbrRec &om, unsigned it, const Consts &co, V3 fb_o, V3 tb_o,
                                        const NbrRec *__restrict__ nbr, const Planes &acc, ItemBar &ib,
                                        ParamBar &ipar) {
  const V3 rl = mk(om.rx, om.ry, om.rz), vl = mk(om.vx, om.vy, om.vz), wl = mk(om.wx, om.wy, om.wz);
  ib = zero_item();
  int k;
  if (it >= kBndItem) {
    const int rt = (int)((it >> 2) & 7u);
    k = (int)(it & 3u);
    Sph q;
    q.r = rl; q.v = vl; q.w = wl;
    q.s = mk(om.s[3 * k], om.s[3 * k + 1], om.s[3 * k + 2]);
    q.rad = om.rad;
    q.mwall = om.mwall;
    wall_rev(rt, q, co, fb_o, tb_o, ib, ipar);
  } else {
    const int t = (int)(it >> 4), p = (int)(it & 15u);
    k = p & 3;
    const int sm = p >> 2;
    const V3 s1 = mk(om.s[3 * k], om.s[3 * k + 1], om.s[3 * k + 2]);
    V3 pr_b, pv_b, pw_b, ps_b;
    bool any;
    pair_rev(rl, vl, wl, s1, om.rad, om.msph, nbr[t], sm, co, co.variant == AF3D_FRICTION_DEV, fb_o, tb_o, ib,
             pr_b, pv_b, pw_b, ps_b, ipar, any);
    if (any) {
      atomic_add3(acc, CR, t, pr_b);
      atomic_add3(acc, CV, t, pv_b);
      atomic_add3(acc, CW, t, pw_b);
      atomic_add3(acc, CS + 3 * sm, t, ps_b);
    }
  }
  return k;
}

__device__ __forceinline__ void add_par(ParamBar &par, const ParamBar &ipar) {
  par.kappa_pp += ipar.kappa_pp; par.gamma_pp += ipar.gamma_pp; par.mu_pp += ipar.mu_pp;
  par.kappa_pw += ipar.kappa_pw; par.gamma_pw += ipar.gamma_pw; par.mu_pw += ipar.mu_pw;
}

// Reverse of finish_Verlet, get_accel and every contact of one clump (startup: the start-up
// force pass, which has no finish and whose accelerations become a_i of the first step).
// in: adjoint of the next state; out.a/out.al receive the finish terms of this step's a_i and
// alpha_i; acc receives (atomically) the adjoints of every clump's r1, v1, w1 and spheres;
// rb receives this clump's own R1 adjoint.  The contacts run warp-cooperatively: the item lists
// of the forward pass, rebuilt here, 32 items a round, each lane reversing one contact for its
// owner.
#ifndef AF3D_ADJ_MINB
#define AF3D_ADJ_MINB 1
#endif
__global__ void __launch_bounds__(kAdjCoopBlock, AF3D_ADJ_MINB) k_adj_forces(Planes P, Planes in, Planes out, Planes acc,
                                                              Planes rb, DevScalars *d, const int *__restrict__ flume,
                                                              const NbrRec *__restrict__ nbr,
                                                              const CullRec *__restrict__ cull,
                                                              const int *__restrict__ start,
                                                              const int *__restrict__ order,
                                                              const float4 *__restrict__ csort, double *param_b,
                                                              int startup, long n) {
  __shared__ AdjQueue queues[kAdjCoopBlock / 32];
  AdjQueue &aq = queues[threadIdx.x >> 5];
  const int lane = threadIdx.x & 31;
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const bool valid = s < n;
  const long sv = valid ? s : n - 1;
  const long wbase = blockIdx.x * (long)blockDim.x + (threadIdx.x & ~31u);
  ParamBar par = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  const int f = flume[sv];
  const Consts &c = d->flumes[f].c;
  const af3d_cell_par g = d->flumes[f].grid;
  const long long off = d->flumes[f].cell_off;
  const NbrRec &me = nbr[sv];
  Own o;
  o.r = mk(me.rx, me.ry, me.rz);
  o.v = mk(me.vx, me.vy, me.vz);
  o.w = mk(me.wx, me.wy, me.wz);
  for (int k = 0; k < 4; k++) o.s[k] = mk(me.s[3 * k], me.s[3 * k + 1], me.s[3 * k + 2]);
  o.rad = me.rad; o.msph = me.msph; o.mwall = me.mwall;
  const bool removed = is_removed(*c.tp, o.r.x, c.side_x);
  const bool act = valid && !removed;
  ClumpBar ob;
  V3 Fb, Tb;
  adj_head(s, act, valid, startup, o, c, P, in, out, rb, ob, Fb, Tb);
  aq.fb[0][lane] = Fb.x; aq.fb[1][lane] = Fb.y; aq.fb[2][lane] = Fb.z;
  aq.fb[3][lane] = Tb.x; aq.fb[4][lane] = Tb.y; aq.fb[5][lane] = Tb.z;
  for (int k = 0; k < 21; k++) aq.own[k][lane] = 0.0;
  // the contacts: the forward pass's item lists, reversed 32 a round
  const bool aval = c.phase == AF3D_PHASE_AVALANCHE;
  const double B = (double)cull[sv].c.w;
  bool slow = false;
  ListCounts lcounts;
  const int nitems = build_item_lists(aq.il.pl, &aq.il.items[0][lane], 32, wbase, sv, act, aval, o.r, c, g,
                                      d->flumes[f].gridf, off, nbr, cull, start, order, csort, slow, lcounts);
  const int total = warp_prefix(nitems, aq.il.base);
  for (int j0 = 0; j0 < total; j0 += 32) {
    const int j = j0 + lane;
    if (j < total) {
      const int lo = owner_of(aq.il.base, j);
      const unsigned it = aq.il.items[j - aq.il.base[lo]][lo];
      const long os = wbase + lo;
      const int of = flume[os];
      const Consts &co = of == f ? c : d->flumes[of].c;
      ItemBar ib;
      ParamBar ipar = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};   // this item's; the lane's flume or the owner's
      const int k = adj_item(nbr[os], it, co, mk(aq.fb[0][lo], aq.fb[1][lo], aq.fb[2][lo]),
                             mk(aq.fb[3][lo], aq.fb[4][lo], aq.fb[5][lo]), nbr, acc, ib, ipar);
      if (of == f) add_par(par, ipar);
      else flush_params(param_b, of, ipar);
      double *ow = &aq.own[0][lo];
      shared_add3(ow + 32 * CR, ib.r);
      shared_add3(ow + 32 * CV, ib.v);
      shared_add3(ow + 32 * CW, ib.w);
      shared_add3(ow + 32 * (CS + 3 * k), ib.s);
    }
  }
  __syncwarp();
  if (act) {
    if (slow) adj_contacts_lane(s, o, c, g, off, B, Fb, Tb, acc, nbr, cull, start, order, ob, par);
    auto own3 = [&](int c0) { return mk(aq.own[c0][lane], aq.own[c0 + 1][lane], aq.own[c0 + 2][lane]); };
    atomic_add3(acc, CR, s, ob.r + own3(CR));
    atomic_add3(acc, CV, s, ob.v + own3(CV));
    atomic_add3(acc, CW, s, ob.w + own3(CW));
    for (int k = 0; k < 4; k++) atomic_add3(acc, CS + 3 * k, s, ob.s[k] + own3(CS + 3 * k));
  }
  add_params(param_b, f, par);
}

// The same reverse from the item lists the forward pass recorded (ContactLists with cnt), pooled
// over a block of 128 clumps: the block's particle items, then its boundary items, 32 a round per
// warp, owners' adjoints summed in shared memory (a reverse needs no order).
constexpr int kAdjListBlock = 128;
struct AdjBlock {
  double fb[6][kAdjListBlock];
  double own[21][kAdjListBlock];
  int base[kAdjListBlock + 1], pbase[kAdjListBlock + 1], qbase[kAdjListBlock + 1];
  int npre[kAdjListBlock];
  int wsum[3][kAdjListBlock / 32];
};

#ifndef AF3D_ADJ_LMINB
#define AF3D_ADJ_LMINB 1
#endif
__global__ void __launch_bounds__(kAdjListBlock, AF3D_ADJ_LMINB) k_adj_forces_l(Planes P, Planes in, Planes out, Planes acc,
                                                               Planes rb, DevScalars *d, const int *__restrict__ flume,
                                                               const NbrRec *__restrict__ nbr,
                                                               const CullRec *__restrict__ cull,
                                                               const int *__restrict__ start,
                                                               const int *__restrict__ order, ContactLists lists,
                                                               double *param_b, long n) {
  __shared__ AdjBlock ab;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long bbase = blockIdx.x * (long)kAdjListBlock;
  const long s = bbase + tid;
  const bool valid = s < n;
  const long sv = valid ? s : n - 1;
  ParamBar par = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  const int f = flume[sv];
  const Consts &c = d->flumes[f].c;
  const NbrRec &me = nbr[sv];
  Own o;
  o.r = mk(me.rx, me.ry, me.rz);
  o.v = mk(me.vx, me.vy, me.vz);
  o.w = mk(me.wx, me.wy, me.wz);
  for (int k = 0; k < 4; k++) o.s[k] = mk(me.s[3 * k], me.s[3 * k + 1], me.s[3 * k + 2]);
  o.rad = me.rad; o.msph = me.msph; o.mwall = me.mwall;
  const bool removed = is_removed(*c.tp, o.r.x, c.side_x);
  const bool act = valid && !removed;
  ClumpBar ob;
  V3 Fb, Tb;
  adj_head(s, act, valid, 0, o, c, P, in, out, rb, ob, Fb, Tb);
  ab.fb[0][tid] = Fb.x; ab.fb[1][tid] = Fb.y; ab.fb[2][tid] = Fb.z;
  ab.fb[3][tid] = Tb.x; ab.fb[4][tid] = Tb.y; ab.fb[5][tid] = Tb.z;
  for (int k = 0; k < 21; k++) ab.own[k][tid] = 0.0;
  // the clump's recorded list layout
  const int packed = act ? lists.cnt[s] : 0;
  const bool slow = act && packed < 0;
  const int nitems = packed > 0 ? (packed & 0xff) : 0;
  const int npre = packed > 0 ? ((packed >> 8) & 0xff) : 0;
  const int npair = packed > 0 ? ((packed >> 16) & 0xff) : 0;
  ab.npre[tid] = npre;
  int v[3] = {nitems, npair, nitems - npair};
#pragma unroll
  for (int q = 0; q < 3; q++) {
    for (int k = 1; k < 32; k <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, v[q], k);
      if (lane >= k) v[q] += u;
    }
    if (lane == 31) ab.wsum[q][warp] = v[q];
  }
  __syncthreads();
  const int own_cnt[3] = {nitems, npair, nitems - npair};
  int *dst[3] = {ab.base, ab.pbase, ab.qbase};
#pragma unroll
  for (int q = 0; q < 3; q++) {
    int wofs = 0, tot = 0;
    for (int w = 0; w < kAdjListBlock / 32; w++) {
      const int t = ab.wsum[q][w];
      wofs += w < warp ? t : 0;
      tot += t;
    }
    dst[q][tid] = wofs + v[q] - own_cnt[q];
    if (tid == kAdjListBlock - 1) dst[q][kAdjListBlock] = tot;
  }
  __syncthreads();
  const int total = ab.base[kAdjListBlock], ptotal = ab.pbase[kAdjListBlock];
  auto owner = [&](const int *b, int j) {
    int lo = 0, hi = kAdjListBlock - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (b[mid] <= j) lo = mid; else hi = mid - 1;
    }
    return lo;
  };
  for (int r0 = warp * 32; r0 < total; r0 += kAdjListBlock) {
    const int i = r0 + lane;
    if (i < total) {
      int lo, idx;
      if (i < ptotal) {
        lo = owner(ab.pbase, i);
        idx = ab.npre[lo] + (i - ab.pbase[lo]);
      } else {
        const int ib = i - ptotal;
        lo = owner(ab.qbase, ib);
        const int b = ib - ab.qbase[lo], np = ab.npre[lo];
        idx = b < np ? b : b + (ab.pbase[lo + 1] - ab.pbase[lo]);
      }
      const unsigned it = lists.items[(long)idx * n + bbase + lo];
      const long os = bbase + lo;
      const int of = flume[os];
      const Consts &co = of == f ? c : d->flumes[of].c;
      ItemBar itb;
      ParamBar ipar = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
      const int k = adj_item(nbr[os], it, co, mk(ab.fb[0][lo], ab.fb[1][lo], ab.fb[2][lo]),
                             mk(ab.fb[3][lo], ab.fb[4][lo], ab.fb[5][lo]), nbr, acc, itb, ipar);
      if (of == f) add_par(par, ipar);
      else flush_params(param_b, of, ipar);
      double *ow = &ab.own[0][lo];
      atomicAdd(ow + kAdjListBlock * CR, itb.r.x); atomicAdd(ow + kAdjListBlock * (CR + 1), itb.r.y);
      atomicAdd(ow + kAdjListBlock * (CR + 2), itb.r.z);
      atomicAdd(ow + kAdjListBlock * CV, itb.v.x); atomicAdd(ow + kAdjListBlock * (CV + 1), itb.v.y);
      atomicAdd(ow + kAdjListBlock * (CV + 2), itb.v.z);
      atomicAdd(ow + kAdjListBlock * CW, itb.w.x); atomicAdd(ow + kAdjListBlock * (CW + 1), itb.w.y);
      atomicAdd(ow + kAdjListBlock * (CW + 2), itb.w.z);
      const int cs = CS + 3 * k;
      atomicAdd(ow + kAdjListBlock * cs, itb.s.x); atomicAdd(ow + kAdjListBlock * (cs + 1), itb.s.y);
      atomicAdd(ow + kAdjListBlock * (cs + 2), itb.s.z);
    }
  }
  __syncthreads();
  if (act) {
    if (slow) {
      const af3d_cell_par g = d->flumes[f].grid;
      adj_contacts_lane(s, o, c, g, d->flumes[f].cell_off, (double)cull[sv].c.w, Fb, Tb, acc, nbr, cull, start,
                        order, ob, par);
    }
    auto own3 = [&](int c0) { return mk(ab.own[c0][tid], ab.own[c0 + 1][tid], ab.own[c0 + 2][tid]); };
    atomic_add3(acc, CR, s, ob.r + own3(CR));
    atomic_add3(acc, CV, s, ob.v + own3(CV));
    atomic_add3(acc, CW, s, ob.w + own3(CW));
    for (int k = 0; k < 4; k++) atomic_add3(acc, CS + 3 * k, s, ob.s[k] + own3(CS + 3 * k));
  }
  add_params(param_b, f, par);
}

// The objectives, per flume f, over its clumps' final downslope positions x = x_rot
// (rotate_vectors.cu:28) with masses m:
//   deposit centroid (length <= 0):  J = sum m x / sum m
//   runout (length l > 0):           J = l ln(sum m exp(x / l) / sum m), the mass-weighted
//                                    soft maximum of x: the front of the deposit as l -> 0, the
//                                    centroid as l -> infinity; evaluated as
//                                    x_max + l ln(sum m exp((x - x_max) / l) / sum m)
// Three sums per flume: sums[3 f] = sum m x (centroid) or sum m exp((x - x_max) / l) (runout),
// sums[3 f + 1] = sum m, sums[3 f + 2] = x_max as an order-preserving integer (runout only;
// zero, below every key, before the first pass).
__device__ __forceinline__ unsigned long long order_key(double x) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(x);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double from_order_key(unsigned long long k) {
  const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

__device__ __forceinline__ double final_xrot(const Planes &P, const af3d_system_par &sy, long s) {
  return P.p[RX][s] * sy.cost - P.p[RZ][s] * sy.sint;
}

// Runout, first pass: x_max per flume.
__global__ void k_adj_xmax(Planes P, DevScalars *d, const int *__restrict__ flume, double *sums, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int f = flume[s];
  atomicMax(reinterpret_cast<unsigned long long *>(sums + 3 * f + 2), order_key(final_xrot(P, d->flumes[f].sys, s)));
}

__global__ void k_adj_objective(Planes P, DevScalars *d, const int *__restrict__ flume, double *sums, double length,
                                long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long sv = s < n ? s : n - 1;
  const int f = flume[sv];
  double mx = 0.0, m = 0.0;
  if (s < n) {
    const double x = final_xrot(P, d->flumes[f].sys, s);
    m = P.p[MASS][s];
    if (length > 0.0) {
      const double xmax = from_order_key(reinterpret_cast<const unsigned long long *>(sums)[3 * f + 2]);
      mx = m * exp((x - xmax) / length);
    } else {
      mx = m * x;
    }
  }
  const int f0 = __shfl_sync(0xffffffffu, f, 0);
  if (__all_sync(0xffffffffu, f == f0)) {
    warp_reduce_add(sums + 3 * f0, mx);
    warp_reduce_add(sums + 3 * f0 + 1, m);
  } else if (s < n) {
    atomicAdd(sums + 3 * f, mx);
    atomicAdd(sums + 3 * f + 1, m);
  }
}

// Seed: the adjoint of the final state for the sum over flumes of J_f (the flumes are
// independent, so each flume's gradients are those of its own J_f): dJ/dx = m / sum m
// (centroid) or m exp((x - x_max) / l) / sum m exp((x - x_max) / l) (runout), and
// dx/dr = (cos, 0, -sin).
__global__ void k_adj_seed(Planes P, Planes adj, DevScalars *d, const int *__restrict__ flume, const double *sums,
                           double length, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  const int f = flume[s];
  const af3d_system_par &sy = d->flumes[f].sys;
  double w;
  if (length > 0.0) {
    const double xmax = from_order_key(reinterpret_cast<const unsigned long long *>(sums)[3 * f + 2]);
    w = P.p[MASS][s] * exp((final_xrot(P, sy, s) - xmax) / length) / sums[3 * f];
  } else {
    w = P.p[MASS][s] / sums[3 * f + 1];
  }
  for (int k = 0; k < NADJ; k++) adj.p[k][s] = 0.0;
  st3(adj, AR, s, mk(w * sy.cost, 0.0, -w * sy.sint));
}

// The state of a step (r, v, w, R, a_i, alpha_i; with spheres also the four sphere centres)
// between the planes and a tape slot.  The steps recompute the sphere centres from r and R; the
// start-up force pass reads them as they are.
// The state planes r, v, w, R, a_i, alpha_i (consecutive in the plane order), then the sphere
// centres (SPHERES), between the plane set and a tape slot; every load is issued before the stores.
static_assert(RX == 0 && R22 == 17 && AIX == 18 && ALIZ == 23, "state planes 0..23 are consecutive");
template <int NP>
__global__ void k_state_copy(Planes P, Planes tape, int to_tape, long n) {
  const long s = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (s >= n) return;
  double v[NP];
#pragma unroll
  for (int k = 0; k < NP; k++) {
    const int p = k < NADJ ? k : S0X + (k - NADJ);
    v[k] = to_tape ? P.p[p][s] : tape.p[k][s];
  }
#pragma unroll
  for (int k = 0; k < NP; k++) {
    const int p = k < NADJ ? k : S0X + (k - NADJ);
    if (to_tape) tape.p[k][s] = v[k];
    else P.p[p][s] = v[k];
  }
}


}  // namespace

void launch_adj_forces(const Launch &L, Planes P, Planes in, Planes out, Planes acc, Planes rb, DevScalars *d,
                       const int *flume, const NbrRec *nbr, const CullRec *cull, const int *start, const int *order,
                       const float4 *csort, double *param_b, bool startup) {
  if (L.n <= 0) return;
  const unsigned nb = (unsigned)((L.n + kAdjCoopBlock - 1) / kAdjCoopBlock);
  k_adj_forces<<<nb, kAdjCoopBlock, 0, L.st>>>(P, in, out, acc, rb, d, flume, nbr, cull, start, order, csort, param_b,
                                               startup ? 1 : 0, L.n);
}

void launch_adj_forces_lists(const Launch &L, Planes P, Planes in, Planes out, Planes acc, Planes rb, DevScalars *d,
                             const int *flume, const NbrRec *nbr, const CullRec *cull, const int *start,
                             const int *order, ContactLists lists, double *param_b) {
  if (L.n <= 0) return;
  const unsigned nb = (unsigned)((L.n + kAdjListBlock - 1) / kAdjListBlock);
  k_adj_forces_l<<<nb, kAdjListBlock, 0, L.st>>>(P, in, out, acc, rb, d, flume, nbr, cull, start, order, lists,
                                                 param_b, L.n);
}

void launch_adj_objective(const Launch &L, Planes P, DevScalars *d, const int *flume, double *sums, double length) {
  if (L.n <= 0) return;
  if (length > 0.0) k_adj_xmax<<<blocks(L.n), kAdjBlock, 0, L.st>>>(P, d, flume, sums, L.n);
  k_adj_objective<<<blocks(L.n), kAdjBlock, 0, L.st>>>(P, d, flume, sums, length, L.n);
}

void launch_adj_seed(const Launch &L, Planes P, Planes adj, DevScalars *d, const int *flume, const double *sums,
                     double length) {
  if (L.n <= 0) return;
  k_adj_seed<<<blocks(L.n), kAdjBlock, 0, L.st>>>(P, adj, d, flume, sums, length, L.n);
}

void launch_state_copy(const Launch &L, Planes P, Planes tape, bool to_tape, bool spheres) {
  if (L.n <= 0) return;
  if (spheres)
    k_state_copy<NADJ + 12><<<blocks(L.n), kAdjBlock, 0, L.st>>>(P, tape, to_tape ? 1 : 0, L.n);
  else
    k_state_copy<NADJ><<<blocks(L.n), kAdjBlock, 0, L.st>>>(P, tape, to_tape ? 1 : 0, L.n);
}

}  // namespace af3d
