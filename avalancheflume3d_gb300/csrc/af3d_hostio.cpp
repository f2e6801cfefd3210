// af3d_hostio.cpp -- host-only parts of the C ABI: DataInput.dat, the derived parameters,
// error_check, last_config.dat, the snapshot files, and the initial-state generators.  No GPU
// involved.
//
// Compiled with -ffp-contract=off so the derived parameters come out bit-identical to the
// reference's start-up arithmetic (avalanche_hst.cu:84-102, 187-195) on any host.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/af3d.h"

namespace {

constexpr double kPI = 3.1415926535897932;   // cabecera.hu:5-19
constexpr double kGRAV = 981.0;
constexpr double kGYR = 4.4494897427831781;
constexpr double kROOT2 = 1.414213562373095;
constexpr double kHOP_HEIGHT = 25.0;
constexpr double kHOP_WIDTH = 15.0;
constexpr double kYFUNNEL = 30.0;
constexpr double kLFUNNEL = 70.0;
constexpr double kYHOP_L = 7.5;
constexpr double kYHOP_R = 22.5;

bool first_token(FILE *fp, const char *fmt, void *out) {
  char row[256];
  if (!fgets(row, sizeof row, fp)) return false;
  return sscanf(row, fmt, out) == 1;
}

}  // namespace

extern "C" {

af3d_status af3d_read_datainput(FILE *fp, af3d_inputs *in) {
  if (!fp || !in) return AF3D_ERR_ARG;
  af3d_inputs v{};
  // avalanche_hst.cu:34-81: the first token of each of 16 lines, in this order.
  bool ok = first_token(fp, "%ld", &v.npart) && first_token(fp, "%lf", &v.width) &&
            first_token(fp, "%lf", &v.hopper_height) && first_token(fp, "%lf", &v.rmin) &&
            first_token(fp, "%lf", &v.rmax) && first_token(fp, "%lf", &v.v0) &&
            first_token(fp, "%lf", &v.dt) && first_token(fp, "%lf", &v.eps_pw) &&
            first_token(fp, "%lf", &v.mu_pw) && first_token(fp, "%lf", &v.eps_pp) &&
            first_token(fp, "%lf", &v.mu_pp) && first_token(fp, "%lf", &v.t_coll) &&
            first_token(fp, "%lf", &v.Lflume) && first_token(fp, "%lf", &v.tilt_deg) &&
            first_token(fp, "%ld", &v.ntags) && first_token(fp, "%d", &v.print_flag);
  if (!ok) return AF3D_ERR_IO;
  *in = v;
  return AF3D_OK;
}

af3d_status af3d_load_datainput(const char *path, af3d_inputs *in) {
  if (!path || !in) return AF3D_ERR_ARG;
  FILE *fp = fopen(path, "r");
  if (!fp) return AF3D_ERR_IO;
  const af3d_status s = af3d_read_datainput(fp, in);
  fclose(fp);
  return s;
}

af3d_status af3d_derive_system(const af3d_inputs *in, af3d_system_par *sys, af3d_funnel *fun) {
  if (!in || !sys || !fun) return AF3D_ERR_ARG;
  af3d_system_par s{};
  s.npart = in->npart;
  s.side.y = in->width;
  s.side.z = in->hopper_height;
  s.rmin = in->rmin;
  s.rmax = in->rmax;
  s.v0 = in->v0;
  s.dt = in->dt;
  s.eps_pw = in->eps_pw;
  s.mu_pw = in->mu_pw;
  s.eps_pp = in->eps_pp;
  s.mu_pp = in->mu_pp;
  s.t_coll = in->t_coll;
  s.Lflume = in->Lflume;
  s.tilt = in->tilt_deg;
  // avalanche_hst.cu:84-94
  s.side.x = kHOP_WIDTH;
  s.time = -1.0;
  s.hdt = 0.5 * s.dt;
  s.tilt *= kPI / 180.0;
  s.gyr_max = kGYR * s.rmax;
  s.sint = sin(s.tilt);
  s.cost = cos(s.tilt);
  s.sintg = kGRAV * s.sint;
  s.costg = kGRAV * s.cost;
  s.xfunnel = kLFUNNEL * s.cost;
  s.dy2 = 0.5 * (kYFUNNEL - s.side.y);
  // avalanche_hst.cu:99-102
  const double hipof = sqrt(s.dy2 * s.dy2 + kLFUNNEL * kLFUNNEL);
  fun->sinfi = s.dy2 / hipof;
  fun->cosfi = kLFUNNEL / hipof;
  fun->tanfi = s.dy2 / kLFUNNEL;
  // avalanche_hst.cu:187-195
  const double aux_0 = kPI / s.t_coll;
  double aux_1 = log(s.eps_pp) / s.t_coll;
  s.gamma_pp = -2.0 * log(s.eps_pp) / s.t_coll;
  s.kappa_pp = (aux_0 * aux_0 + aux_1 * aux_1);
  aux_1 = log(s.eps_pw) / s.t_coll;
  s.gamma_pw = -2.0 * log(s.eps_pw) / s.t_coll;
  s.kappa_pw = (aux_0 * aux_0 + aux_1 * aux_1);
  s.fr_fact_pp = s.mu_pp / 1.0e12;
  s.fr_fact_pw = s.mu_pw / 1.0e12;
  *sys = s;
  return AF3D_OK;
}

int af3d_error_check(const af3d_system_par *s, char *msg, size_t msglen) {
  // error_check.cu:7-63: every failing check overwrites the number; the last one wins.
  int errn = 0;
  std::string m;
  char buf[256];
  if (s->npart <= 0) {
    snprintf(buf, sizeof buf, "ERROR. No particles in box! n = %ld\n", s->npart);
    m = buf; errn = 1;
  }
  if (s->side.x <= 0.0 || s->side.y <= 0.0 || s->side.z <= 0.0) {
    snprintf(buf, sizeof buf, "ERROR. Wrong box dimensions. x = %lf, y = %lf, z = %lf\n", s->side.x,
             s->side.y, s->side.z);
    m = buf; errn = 2;
  }
  if (s->rmin <= 0.0 || s->rmax <= 0.0) {
    snprintf(buf, sizeof buf, "ERROR. Wrong sphere radius. rmax = %lf, rmin = %lf\n", s->rmax, s->rmin);
    m = buf; errn = 3;
  }
  if (s->rmax < s->rmin) {
    snprintf(buf, sizeof buf, "ERROR rmax must be larger than rmin. rmax = %lf, rmin = %lf\n", s->rmax,
             s->rmin);
    m = buf; errn = 4;
  }
  if (s->eps_pw <= 0.0 || s->eps_pw > 1.0) { m = "ERROR. eps_pw must be 0 < eps_pw <= 1\n"; errn = 5; }
  if (s->eps_pp <= 0.0 || s->eps_pp > 1.0) { m = "ERROR. eps_pp must be 0 < eps_pp <= 1\n"; errn = 6; }
  if (s->mu_pw < 0.0 || s->mu_pw > 1.0) { m = "ERROR. mu_pw must be 0 < mu_pw < 1\n"; errn = 7; }
  if (s->mu_pp < 0.0 || s->mu_pp > 1.5) { m = "ERROR. mu_pp must be 0 < mu_pp < 1\n"; errn = 8; }
  if (tan(s->tilt) < 1.25 * s->mu_pw) {
    m = "ERROR. Particles won't go down the slope.\n Please, increase tilt or reduce mu_pw.\n";
    errn = 9;
  }
  if (msg && msglen) {
    strncpy(msg, m.c_str(), msglen - 1);
    msg[msglen - 1] = '\0';
  }
  return errn;
}

af3d_status af3d_write_last_config(const char *path, int aval_start, double time, long cc, long jj,
                                   const af3d_particle *pp, long n) {
  // avalanche_hst.cu:519-548 (header aval_start, time, cc, jj; then id r R v w per clump, %lf)
  FILE *fp = fopen(path, "w");
  if (!fp) return AF3D_ERR_IO;
  fprintf(fp, "%d\n%lf\n%ld\n%ld\n", aval_start, time, cc, jj);
  for (long i = 0; i < n; i++) {
    const af3d_particle &p = pp[i];
    fprintf(fp, "%ld %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf\n", i,
            p.rr.x, p.rr.y, p.rr.z, p.Rmatx.x, p.Rmatx.y, p.Rmatx.z, p.Rmaty.x, p.Rmaty.y, p.Rmaty.z,
            p.Rmatz.x, p.Rmatz.y, p.Rmatz.z, p.vv.x, p.vv.y, p.vv.z, p.ww.x, p.ww.y, p.ww.z);
  }
  return fclose(fp) == 0 ? AF3D_OK : AF3D_ERR_IO;
}

af3d_status af3d_append_snapshot(const char *xyz_path, const char *vel_path, const char *vmean_path,
                                 const char *xcm_path, const af3d_particle *pp, long n,
                                 const af3d_system_par *sys, int phase) {
  // avalanche_hst.cu:507-586 (fill phase) and :750-841 (avalanche phase), one output frame
  if (!sys || n < 0 || (n > 0 && !pp)) return AF3D_ERR_ARG;
  const bool aval = phase == AF3D_PHASE_AVALANCHE;
  const double xfinal = (kLFUNNEL + sys->Lflume) * sys->cost;   // avalanche_hst.cu:116
  auto open = [](const char *path, FILE **fp) {
    *fp = path ? fopen(path, "a") : nullptr;
    return !path || *fp;
  };
  FILE *xyz, *vel, *vm, *xc;
  if (!open(xyz_path, &xyz)) return AF3D_ERR_IO;
  if (!open(vel_path, &vel)) {
    if (xyz) fclose(xyz);
    return AF3D_ERR_IO;
  }
  if (!open(vmean_path, &vm)) {
    if (xyz) fclose(xyz);
    if (vel) fclose(vel);
    return AF3D_ERR_IO;
  }
  if (!open(aval ? xcm_path : nullptr, &xc)) {
    if (xyz) fclose(xyz);
    if (vel) fclose(vel);
    if (vm) fclose(vm);
    return AF3D_ERR_IO;
  }
  if (xyz) fprintf(xyz, "%ld\n\n", 4 * n + 2);
  if (vel) fprintf(vel, "%ld\n\n", n + 2);
  double vmean = 0.0, wmean = 0.0;
  for (long i = 0; i < n; i++) {
    const af3d_particle &p = pp[i];
    if (xyz)
      for (int k = 0; k < 4; k++)
        fprintf(xyz, "%lf %lf %lf %lf %ld\n", p.radius, p.rr_s[k].x, p.rr_s[k].y, p.rr_s[k].z, i);
    if (vel) fprintf(vel, "%lf %lf %lf %lf %lf %ld\n", p.rr.x, p.rr.y, p.rr.z, p.vv.x, p.ww.y, i);
    double vm2 = p.vv.x * p.vv.x;
    vm2 += p.vv.y * p.vv.y;
    vm2 += p.vv.z * p.vv.z;
    vmean += std::sqrt(vm2);
    double wm2 = p.ww.x * p.ww.x;
    wm2 += p.ww.y * p.ww.y;
    wm2 += p.ww.z * p.ww.z;
    wmean += std::sqrt(wm2);
  }
  // ghost atoms that keep the rendered cell size constant
  if (xyz) {
    if (aval)
      fprintf(xyz, "0.0001 %lf %lf %lf %ld\n", sys->side.x, kYFUNNEL, sys->side.z, n);
    else
      fprintf(xyz, "0.000001 %lf %lf %lf %ld\n", xfinal, kYFUNNEL, sys->side.z, n);
    fprintf(xyz, "0.000001 0.000000 0.000000 0.000000 %ld\n", n);
  }
  if (vel) {
    fprintf(vel, "%lf %lf %lf 0.000000 0.000000 %ld\n", xfinal, kYFUNNEL, sys->side.z, n);
    fprintf(vel, "0.000000 0.000000 0.000000 0.000000 0.000000 %ld\n", n);
  }
  vmean /= n;
  wmean /= n;
  if (vm) fprintf(vm, "%lf, %lf, %lf\n", sys->time - sys->dt, vmean, wmean);
  if (xc) {
    double xcm = 0.0, zcm = 0.0;
    for (long i = 0; i < n; i++) {
      const double xmass = pp[i].mass * pp[i].rr.x;
      const double zmass = pp[i].mass * pp[i].rr.z;
      xcm += xmass;
      zcm += zmass;
    }
    xcm /= sys->tot_mass;
    zcm /= sys->tot_mass;
    fprintf(xc, "%lf, %lf, %lf\n", sys->time - sys->dt, xcm, zcm);
  }
  bool ok = true;
  for (FILE *f : {xyz, vel, vm, xc})
    if (f) ok = fclose(f) == 0 && ok;
  return ok ? AF3D_OK : AF3D_ERR_IO;
}

af3d_status af3d_read_last_config(const char *path, int *aval_start, double *time, long *cc, long *jj,
                                  af3d_particle *pp, long n) {
  // avalanche_hst.cu:224-293: header, then `id` and 18 values per line; sphere centres are
  // recomputed from the stored r, R and the radius already in pp.
  FILE *fp = fopen(path, "r");
  if (!fp) return AF3D_ERR_IO;
  if (fscanf(fp, "%d\n", aval_start) != 1 || fscanf(fp, "%lf\n", time) != 1 ||
      fscanf(fp, "%ld\n", cc) != 1 || fscanf(fp, "%ld\n", jj) != 1) {
    fclose(fp);
    return AF3D_ERR_IO;
  }
  long seen = 0;
  for (;;) {
    long i;
    if (fscanf(fp, "%ld ", &i) != 1) break;
    if (i < 0 || i >= n) {
      fclose(fp);
      return AF3D_ERR_IO;
    }
    af3d_particle &p = pp[i];
    int got = fscanf(fp, "%lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf %lf\n",
                     &p.rr.x, &p.rr.y, &p.rr.z, &p.Rmatx.x, &p.Rmatx.y, &p.Rmatx.z, &p.Rmaty.x,
                     &p.Rmaty.y, &p.Rmaty.z, &p.Rmatz.x, &p.Rmatz.y, &p.Rmatz.z, &p.vv.x, &p.vv.y,
                     &p.vv.z, &p.ww.x, &p.ww.y, &p.ww.z);
    if (got != 18) {
      fclose(fp);
      return AF3D_ERR_IO;
    }
    seen++;
  }
  fclose(fp);
  if (seen != n) return AF3D_ERR_IO;
  af3d_sphere_centres(pp, n);
  return AF3D_OK;
}

// ---- generators ----

void af3d_rng_seed(af3d_rng *g, long idum) {
  // rannew64.cu:68-97: 1000 warm-up steps of a 64-bit LCG, then NP = 250 lags from it.
  if (idum < 0) idum = -idum;
  uint64_t u = (uint64_t)idum;
  const uint64_t a = 6364136223846793005ull, c = 1442695040888963407ull;
  for (int i = 0; i < 1000; i++) u = u * a + c;
  for (int i = 0; i < 250; i++) {
    u = u * a + c;
    g->seed[i] = u;
  }
  g->uy = u;
  g->np = 249;
  g->nq = 102;
  g->init = 1;
}

double af3d_rng_next(af3d_rng *g) {
  // rannew64.cu:99-125: lagged Fibonacci x(n) = x(n-250) - x(n-103), an LCG y, return (x-y)/2^64.
  const uint64_t ux = g->seed[g->np] - g->seed[g->nq];
  g->seed[g->np] = ux;
  if (--g->np < 0) g->np = 249;
  if (--g->nq < 0) g->nq = 249;
  g->uy = 2862933555777941757ull * g->uy + 3037000493ull;
  const uint64_t uu = ux - g->uy;
  const double omm = 1.0 / 18446744073709551615.0;
  return omm * (double)uu;
}

void af3d_generate_particles(af3d_particle *pp, const af3d_system_par *sys) {
  for (long i = 0; i < sys->npart; i++) {
    pp[i].density = 2.6;
    pp[i].radius = (i % 20) ? sys->rmin : sys->rmax;
  }
}

void af3d_calculate_particle_parameters(af3d_particle *pp, long n) {
  const double aux1 = 4.0 * kPI / 3.0, aux2 = 112.0 * kPI / 15.0;
  for (long i = 0; i < n; i++) {
    const double rad = pp[i].radius, rho = pp[i].density;
    const double rad3 = rad * rad * rad, rad5 = rad3 * rad * rad;
    pp[i].mass = 4.0 * aux1 * rad3 * rho;
    const double I = aux2 * rho * rad5;
    pp[i].moment_of_inertia = {I, I, I};
  }
}

af3d_status af3d_place_particles(const af3d_system_par *sys, af3d_particle *pp) {
  const double rmax = sys->rmax;
  const double dist = 2.0 + kROOT2 + 0.05 * rmax, hdist = dist / 2.0;
  int ii = 0, jj = 0, kk = 0;
  (void)jj;
  (void)kk;
  for (long a = 0; a < sys->npart; a++) {
    af3d_vec3 r;
    r.x = hdist * rmax + (double)ii * dist * rmax;
    r.y = hdist * rmax + (double)jj * dist * rmax + 0.5 * rmax + kYHOP_L;
    r.z = hdist * rmax + (double)kk * dist * rmax + 0.5 * rmax;
    ii++;
    if (r.x >= sys->side.x - hdist * rmax) {
      r.x = hdist * rmax;
      r.y += dist * rmax;
      jj++;
      ii = 1;
      if (r.y >= kYHOP_R - hdist * rmax) {
        r.y = hdist * rmax + 0.5 * rmax + kYHOP_L;
        r.z += dist * rmax;
        kk++;
        jj = 0;
        if (r.z >= sys->side.z - hdist * rmax) return AF3D_ERR_INPUT;
      }
    }
    r.z += kHOP_HEIGHT;
    const double pos = pp[a].radius / kROOT2;
    af3d_particle &p = pp[a];
    p.rr = r;
    p.rr_s[0] = {r.x + pos, r.y + pos, r.z + pos};
    p.rr_s[1] = {r.x + pos, r.y - pos, r.z - pos};
    p.rr_s[2] = {r.x - pos, r.y - pos, r.z + pos};
    p.rr_s[3] = {r.x - pos, r.y + pos, r.z - pos};
    p.Rmatx = {1.0, 0.0, 0.0};
    p.Rmaty = {0.0, 1.0, 0.0};
    p.Rmatz = {0.0, 0.0, 1.0};
  }
  return AF3D_OK;
}

void af3d_set_initial_velocity(const af3d_system_par *sys, af3d_particle *pp) {
  af3d_rng g;
  af3d_rng_seed(&g, 26752658);
  const double v0 = sys->v0, inv_rm = 1.0 / (4.0 * sys->rmax);
  for (long i = 0; i < sys->npart; i++) {
    const double r0 = 2.0 * kPI * af3d_rng_next(&g) - kPI;
    const double r1 = kPI * af3d_rng_next(&g);
    pp[i].vv = {v0 * cos(r0) * cos(r1), v0 * sin(r0) * cos(r1), v0 * sin(r1)};
    pp[i].ww = {inv_rm * v0 * cos(r0) * cos(r1), inv_rm * v0 * sin(r0) * cos(r1), inv_rm * v0 * sin(r1)};
  }
}

void af3d_sphere_centres(af3d_particle *pp, long n) {
  for (long i = 0; i < n; i++) {
    af3d_particle &p = pp[i];
    const double pos = p.radius / kROOT2;
    const af3d_vec3 r = p.rr, X = p.Rmatx, Y = p.Rmaty, Z = p.Rmatz;
    p.rr_s[0] = {r.x + pos * (X.x + X.y + X.z), r.y + pos * (Y.x + Y.y + Y.z), r.z + pos * (Z.x + Z.y + Z.z)};
    p.rr_s[1] = {r.x + pos * (X.x - X.y - X.z), r.y + pos * (Y.x - Y.y - Y.z), r.z + pos * (Z.x - Z.y - Z.z)};
    p.rr_s[2] = {r.x + pos * (-X.x - X.y + X.z), r.y + pos * (-Y.x - Y.y + Y.z), r.z + pos * (-Z.x - Z.y + Z.z)};
    p.rr_s[3] = {r.x + pos * (-X.x + X.y - X.z), r.y + pos * (-Y.x + Y.y - Y.z), r.z + pos * (-Z.x + Z.y - Z.z)};
  }
}

long af3d_lattice_block(af3d_particle *pp, long n, af3d_vec3 lo, af3d_vec3 hi, double pitch,
                        af3d_rng *rng, int max_tries) {
  const long nx = (long)floor((hi.x - lo.x) / pitch), ny = (long)floor((hi.y - lo.y) / pitch);
  if (nx <= 0 || ny <= 0) return 0;
  const long nz = (long)floor((hi.z - lo.z) / pitch);
  const long cap = nx * ny * (nz > 0 ? nz : 0);
  const long m = n < cap ? n : cap;
  for (long a = 0; a < m; a++) {
    const long i = a % nx, j = (a / nx) % ny, k = a / (nx * ny);
    af3d_particle &p = pp[a];
    p.rr = {lo.x + (i + 0.5) * pitch, lo.y + (j + 0.5) * pitch, lo.z + (k + 0.5) * pitch};
    for (int t = 0; t < (max_tries > 0 ? max_tries : 1); t++) {
      // Shoemake: uniform unit quaternion from three uniforms.
      const double u1 = af3d_rng_next(rng), u2 = af3d_rng_next(rng), u3 = af3d_rng_next(rng);
      const double s1 = sqrt(1.0 - u1), s2 = sqrt(u1);
      const double w = s1 * sin(2 * kPI * u2), x = s1 * cos(2 * kPI * u2);
      const double y = s2 * sin(2 * kPI * u3), z = s2 * cos(2 * kPI * u3);
      p.Rmatx = {1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)};
      p.Rmaty = {2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)};
      p.Rmatz = {2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)};
      af3d_sphere_centres(&p, 1);
      bool bad = false;
      for (int s = 0; s < 4 && !bad; s++) {
        const af3d_vec3 c = p.rr_s[s];
        bad = c.x - p.radius < lo.x || c.x + p.radius > hi.x || c.y - p.radius < lo.y ||
              c.y + p.radius > hi.y || c.z - p.radius < lo.z;
      }
      // overlap with the already placed lattice neighbours (i-1, j-1, k-1 faces and edges)
      for (long di = -1; di <= 1 && !bad; di++)
        for (long dj = -1; dj <= 1 && !bad; dj++)
          for (long dk = -1; dk <= 0 && !bad; dk++) {
            const long ii = i + di, jj2 = j + dj, kk = k + dk;
            if (ii < 0 || jj2 < 0 || kk < 0 || ii >= nx || jj2 >= ny) continue;
            const long b = ii + nx * (jj2 + ny * kk);
            if (b >= a) continue;
            const af3d_particle &q = pp[b];
            for (int s = 0; s < 4 && !bad; s++)
              for (int u = 0; u < 4 && !bad; u++) {
                const double dx = p.rr_s[s].x - q.rr_s[u].x, dy = p.rr_s[s].y - q.rr_s[u].y,
                             dz = p.rr_s[s].z - q.rr_s[u].z, sep = p.radius + q.radius;
                bad = dx * dx + dy * dy + dz * dz < sep * sep;
              }
          }
      if (!bad) break;
    }
    p.vv = {0.0, 0.0, 0.0};
    p.ww = {0.0, 0.0, 0.0};
  }
  return m;
}

long af3d_lattice_pile(af3d_particle *pp, long n, af3d_vec3 lo, af3d_vec3 hi, double pitch,
                       double overlap, af3d_rng *rng, int max_tries) {
  // Columns of a square lattice in x-y; clumps are dropped layer by layer.  Each clump gets a
  // random orientation that keeps its spheres inside the box walls (redrawn up to max_tries),
  // and is then lowered straight down until one of its spheres touches a sphere already placed
  // in its own or a neighbouring column (or the floor z = lo.z), and pressed `overlap` further.
  const long nx = (long)floor((hi.x - lo.x) / pitch), ny = (long)floor((hi.y - lo.y) / pitch);
  if (nx <= 0 || ny <= 0 || n <= 0) return 0;
  const long ncol = nx * ny;
  // the last two clumps dropped into every column (obstacles for the next ones)
  std::vector<long> top(2 * ncol, -1);
  for (long a = 0; a < n; a++) {
    const long col = a % ncol, i = col % nx, j = col / nx;
    af3d_particle &p = pp[a];
    const double cx = lo.x + (i + 0.5) * pitch, cy = lo.y + (j + 0.5) * pitch;
    p.rr = {cx, cy, 0.0};
    for (int t = 0; t < (max_tries > 0 ? max_tries : 1); t++) {
      const double u1 = af3d_rng_next(rng), u2 = af3d_rng_next(rng), u3 = af3d_rng_next(rng);
      const double s1 = sqrt(1.0 - u1), s2 = sqrt(u1);
      const double w = s1 * sin(2 * kPI * u2), x = s1 * cos(2 * kPI * u2);
      const double y = s2 * sin(2 * kPI * u3), z = s2 * cos(2 * kPI * u3);
      p.Rmatx = {1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)};
      p.Rmaty = {2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)};
      p.Rmatz = {2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)};
      af3d_sphere_centres(&p, 1);
      bool bad = false;
      for (int k = 0; k < 4 && !bad; k++)
        bad = p.rr_s[k].x - p.radius < lo.x || p.rr_s[k].x + p.radius > hi.x ||
              p.rr_s[k].y - p.radius < lo.y || p.rr_s[k].y + p.radius > hi.y;
      if (!bad) break;
    }
    // lowest centre height at which no sphere is below the floor or inside a placed sphere
    double zc = -1e300;
    for (int k = 0; k < 4; k++) zc = fmax(zc, lo.z + p.radius - (p.rr_s[k].z - p.rr.z));
    for (long di = -1; di <= 1; di++)
      for (long dj = -1; dj <= 1; dj++) {
        const long ii = i + di, jj = j + dj;
        if (ii < 0 || jj < 0 || ii >= nx || jj >= ny) continue;
        for (int h = 0; h < 2; h++) {
          const long b = top[2 * (ii + nx * jj) + h];
          if (b < 0) continue;
          const af3d_particle &q = pp[b];
          for (int k = 0; k < 4; k++)
            for (int u = 0; u < 4; u++) {
              const double dx = (p.rr_s[k].x) - q.rr_s[u].x, dy = (p.rr_s[k].y) - q.rr_s[u].y;
              const double sep = p.radius + q.radius, h2 = sep * sep - dx * dx - dy * dy;
              if (h2 <= 0.0) continue;
              zc = fmax(zc, q.rr_s[u].z + sqrt(h2) - (p.rr_s[k].z - p.rr.z));
            }
        }
      }
    p.rr.z = zc - overlap;
    af3d_sphere_centres(&p, 1);
    top[2 * col + 1] = top[2 * col];
    top[2 * col] = a;
    p.vv = {0.0, 0.0, 0.0};
    p.ww = {0.0, 0.0, 0.0};
    if (p.rr.z > hi.z) return a;
  }
  return n;
}

}  // extern "C"
