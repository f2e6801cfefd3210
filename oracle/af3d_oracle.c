/*
 * af3d_oracle.c -- CPU oracle for the AvalancheFlume3D clump-DEM step.
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker of tests/ and the timed CPU
 * baseline of bench.py.  It is never part of the product path.
 *
 * A restatement of the reference's host step routines.  Each function cites
 * the reference file:line it follows.  The arithmetic of every expression
 * keeps the reference's evaluation order; the file must be compiled with
 * -ffp-contract=off (oracle/build.py does) so that no multiply-add is fused.
 * Parity is pinned against the reference compiled from source
 * (tests/test_oracle_pin.py) and against tests/golden/.
 *
 * Structure differs from the reference on purpose: one contact-law helper
 * serves every contact type, spheres are addressed as arrays, and the
 * per-clump loops can run on several host threads (each clump writes only
 * its own force/torque/state entries, exactly as in the reference).
 */
#include "af3d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Constants of cabecera.hu:5-19 (same literals: they fix the arithmetic). */
#define ORC_PI        3.1415926535897932
#define ORC_GRAV      981.0
#define ORC_GYR       4.4494897427831781
#define ORC_SPH_FACT  4.188790204786391
#define ORC_ROOT2     1.414213562373095
#define ORC_DRAG      1.895e-3
#define ORC_HOP_HEIGHT 25.0
#define ORC_HOP_WIDTH  15.0
#define ORC_YFUNNEL    30.0
#define ORC_LFUNNEL    70.0
#define ORC_YHOP_L      7.5
#define ORC_YHOP_R     22.5

static int g_threads = 1;

void orc_set_threads (int nthreads)
{
  g_threads = nthreads > 0 ? nthreads : 1;
#ifdef _OPENMP
  omp_set_num_threads (g_threads);
#endif
}

#ifdef _OPENMP
#define ORC_PARALLEL_FOR _Pragma ("omp parallel for schedule(static) if (g_threads > 1)")
#else
#define ORC_PARALLEL_FOR
#endif

static inline int removed (const orc_system_par *sys, orc_real x)
{
  /* init_Verlet.cu:29, cells.cu:65, force_part.cu:47, ... */
  return sys->time > 0.0 && x > sys->side.x;
}

/*
 * Linear spring-dashpot normal force plus Cundall-Strack tangential force with
 * the reference's Coulomb cap.  This is the common tail of every contact type:
 * force_part.cu:189-241, force_walls.cu:123-177, force_flume.cu:106-160,
 * force_hop.cu:170-224, force_funnel.cu:137-191 and :332-386.
 *
 *   dvvc   relative velocity (partner minus own) at the contact point
 *   nvec   unit normal pointing from the own sphere to the partner
 *   comp   compression (overlap)
 *   km, gm spring and damping coefficients already multiplied by the mass
 *   mass_t mass used by the tangential law (own sphere mass)
 *   xi0    1: the Coulomb branch is also taken when xi was zeroed (walls and
 *          the device particle variant); 0: host particle variant
 *   gate   0: proceed when normal > 0;  1: proceed unless normal <= 0
 *          (force_funnel.cu:354, only differs for a NaN normal)
 * Returns 1 and writes *fs when the contact exerts a force.
 */
static inline int contact_law (orc_vec3 dvvc, orc_vec3 nvec, orc_real comp, orc_real km, orc_real gm,
                               orc_real mass_t, orc_real mu, orc_real cns_1, orc_real dt, int xi0, int gate,
                               orc_vec3 *fs)
{
  orc_real   vn, vt_mag, vt_sig, normal, xi, xi_dot, fsdt, af, t0;
  orc_vec3 vt, tv, f;

  vn   = dvvc.x*nvec.x + dvvc.y*nvec.y + dvvc.z*nvec.z;
  vt.x = dvvc.x - vn*nvec.x;
  vt.y = dvvc.y - vn*nvec.y;
  vt.z = dvvc.z - vn*nvec.z;
  vt_mag = sqrt (vt.x*vt.x + vt.y*vt.y + vt.z*vt.z);
  tv.x = vt.x/vt_mag;
  tv.y = vt.y/vt_mag;
  tv.z = vt.z/vt_mag;
  vt_sig = dvvc.x*tv.x + dvvc.y*tv.y + dvvc.z*tv.z;

  normal = km*comp + gm*(-vn);
  if (gate ? (normal <= 0.0) : !(normal > 0.0))
    return 0;

  f.x = -normal*nvec.x;
  f.y = -normal*nvec.y;
  f.z = -normal*nvec.z;

  xi = dt*vt_sig;
  if (cns_1*normal < fabs (xi))
    xi = 0.0;
  xi_dot = xi/dt;
  fsdt = 1.0e12*mass_t*xi + 2.0e6*mass_t*xi_dot;
  if (vt_mag > 0.0)
  {
    if (fabs (fsdt) > mu*normal || (xi0 && xi == 0.0))
    {
      af  = 0.8*mu*normal/vt_mag;
      t0  = mass_t/af;
      af /= (1.0 + (dt/t0)*(dt/t0));
      f.x += af*vt.x;
      f.y += af*vt.y;
      f.z += af*vt.z;
    }
    else
    {
      if (vt.x != 0.0) f.x += fsdt*vt.x/vt_mag;
      if (vt.y != 0.0) f.y += fsdt*vt.y/vt_mag;
      if (vt.z != 0.0) f.z += fsdt*vt.z/vt_mag;
    }
  }
  *fs = f;
  return 1;
}

/* Velocity of a rigid body point: v + w x (c - r), in the reference's operand order
   (force_part.cu:175-177). */
static inline orc_vec3 point_velocity (orc_vec3 v, orc_vec3 w, orc_vec3 c, orc_vec3 r)
{
  orc_vec3 u;
  u.x = v.x + w.y*(c.z - r.z) - w.z*(c.y - r.y);
  u.y = v.y + w.z*(c.x - r.x) - w.x*(c.z - r.z);
  u.z = v.z + w.x*(c.y - r.y) - w.y*(c.x - r.x);
  return u;
}

/* Accumulate one contact into (F, T) of the clump centred at r (force_part.cu:245-251). */
static inline void accumulate (orc_vec3 *ff, orc_vec3 *tq, orc_vec3 fs, orc_vec3 c, orc_vec3 r)
{
  tq->x += (c.y - r.y)*fs.z - (c.z - r.z)*fs.y;
  tq->y += (c.z - r.z)*fs.x - (c.x - r.x)*fs.z;
  tq->z += (c.x - r.x)*fs.y - (c.y - r.y)*fs.x;
  ff->x += fs.x;
  ff->y += fs.y;
  ff->z += fs.z;
}

/* Wall contact: relative velocity is minus the sphere's contact-point velocity
   (force_walls.cu:113-120).  Returns 1 when a force was added. */
static inline int wall_contact (const orc_particle *p, orc_vec3 rrc, orc_vec3 nvec, orc_real comp,
                                orc_real km, orc_real gm, orc_real mass, orc_real mu, orc_real cns_1, orc_real dt,
                                int gate, orc_vec3 *ff, orc_vec3 *tq)
{
  orc_vec3 vvc, dvvc, fs;
  vvc = point_velocity (p->vv, p->ww, rrc, p->rr);
  dvvc.x = -vvc.x;
  dvvc.y = -vvc.y;
  dvvc.z = -vvc.z;
  if (!contact_law (dvvc, nvec, comp, km, gm, mass, mu, cns_1, dt, 1, gate, &fs))
    return 0;
  accumulate (ff, tq, fs, rrc, p->rr);
  return 1;
}

/* ============================== integration ============================== */

/* init_Verlet.cu:11-152 */
void orc_init_verlet (const orc_vec3 *accel, const orc_vec3 *ang_acc, const orc_system_par *sys,
                      orc_particle *pp)
{
  const long   n   = sys->npart;
  const orc_real dt  = sys->dt;
  const orc_real hdt = sys->hdt;
  long ii;

  ORC_PARALLEL_FOR
  for (ii = 0; ii < n; ii++)
  {
    orc_particle *p = &pp[ii];
    orc_vec3 rr = p->rr, vv, aa, Rx, Ry, Rz, ww, al, dO, u, dRx, dRy, dRz, Tx, Ty, Tz;
    orc_real   mag, c, s, omc, norm, pos;

    if (removed (sys, rr.x))
    {
      p->radius = 0.0;
      continue;
    }
    vv = p->vv;  aa = accel[ii];  ww = p->ww;  al = ang_acc[ii];
    Rx = p->Rmatx;  Ry = p->Rmaty;  Rz = p->Rmatz;

    rr.x += dt*(vv.x + hdt*aa.x);
    rr.y += dt*(vv.y + hdt*aa.y);
    rr.z += dt*(vv.z + hdt*aa.z);
    vv.x += dt*aa.x;
    vv.y += dt*aa.y;
    vv.z += dt*aa.z;

    dO.x = dt*(ww.x + hdt*al.x);
    dO.y = dt*(ww.y + hdt*al.y);
    dO.z = dt*(ww.z + hdt*al.z);
    mag  = sqrt (dO.x*dO.x + dO.y*dO.y + dO.z*dO.z);
    if (mag > 0.0)
    {
      /* Rodrigues rotation about u = dO/|dO| by |dO| (init_Verlet.cu:63-83). */
      u.x = dO.x/mag;  u.y = dO.y/mag;  u.z = dO.z/mag;
      c   = cos (mag);
      s   = sin (mag);
      omc = 1.0 - c;
      dRx.x = omc*u.x*u.x + c;      dRx.y = omc*u.x*u.y - s*u.z;  dRx.z = omc*u.x*u.z + s*u.y;
      dRy.x = omc*u.y*u.x + s*u.z;  dRy.y = omc*u.y*u.y + c;      dRy.z = omc*u.y*u.z - s*u.x;
      dRz.x = omc*u.z*u.x - s*u.y;  dRz.y = omc*u.z*u.y + s*u.x;  dRz.z = omc*u.z*u.z + c;
    }
    else
    {
      dRx.x = 1.0; dRx.y = 0.0; dRx.z = 0.0;
      dRy.x = 0.0; dRy.y = 1.0; dRy.z = 0.0;
      dRz.x = 0.0; dRz.y = 0.0; dRz.z = 1.0;
    }

    /* R <- dR R, rows stored as Rmatx/y/z (init_Verlet.cu:92-100). */
    Tx.x = dRx.x*Rx.x + dRx.y*Ry.x + dRx.z*Rz.x;
    Tx.y = dRx.x*Rx.y + dRx.y*Ry.y + dRx.z*Rz.y;
    Tx.z = dRx.x*Rx.z + dRx.y*Ry.z + dRx.z*Rz.z;
    Ty.x = dRy.x*Rx.x + dRy.y*Ry.x + dRy.z*Rz.x;
    Ty.y = dRy.x*Rx.y + dRy.y*Ry.y + dRy.z*Rz.y;
    Ty.z = dRy.x*Rx.z + dRy.y*Ry.z + dRy.z*Rz.z;
    Tz.x = dRz.x*Rx.x + dRz.y*Ry.x + dRz.z*Rz.x;
    Tz.y = dRz.x*Rx.y + dRz.y*Ry.y + dRz.z*Rz.y;
    Tz.z = dRz.x*Rx.z + dRz.y*Ry.z + dRz.z*Rz.z;

    /* Each column renormalised independently (init_Verlet.cu:103-114). */
    norm = sqrt (Tx.x*Tx.x + Ty.x*Ty.x + Tz.x*Tz.x);
    Rx.x = Tx.x/norm;  Ry.x = Ty.x/norm;  Rz.x = Tz.x/norm;
    norm = sqrt (Tx.y*Tx.y + Ty.y*Ty.y + Tz.y*Tz.y);
    Rx.y = Tx.y/norm;  Ry.y = Ty.y/norm;  Rz.y = Tz.y/norm;
    norm = sqrt (Tx.z*Tx.z + Ty.z*Ty.z + Tz.z*Tz.z);
    Rx.z = Tx.z/norm;  Ry.z = Ty.z/norm;  Rz.z = Tz.z/norm;

    ww.x += dt*al.x;
    ww.y += dt*al.y;
    ww.z += dt*al.z;

    p->rr = rr;  p->vv = vv;  p->ww = ww;
    p->Rmatx = Rx;  p->Rmaty = Ry;  p->Rmatz = Rz;

    /* Sphere centres r + (radius/sqrt2) R s, s in {(+++), (+--), (--+), (-+-)} (init_Verlet.cu:130-142). */
    pos = p->radius/ORC_ROOT2;
    p->rr_s[0].x = rr.x + pos*(Rx.x + Rx.y + Rx.z);
    p->rr_s[0].y = rr.y + pos*(Ry.x + Ry.y + Ry.z);
    p->rr_s[0].z = rr.z + pos*(Rz.x + Rz.y + Rz.z);
    p->rr_s[1].x = rr.x + pos*(Rx.x - Rx.y - Rx.z);
    p->rr_s[1].y = rr.y + pos*(Ry.x - Ry.y - Ry.z);
    p->rr_s[1].z = rr.z + pos*(Rz.x - Rz.y - Rz.z);
    p->rr_s[2].x = rr.x + pos*(-Rx.x - Rx.y + Rx.z);
    p->rr_s[2].y = rr.y + pos*(-Ry.x - Ry.y + Ry.z);
    p->rr_s[2].z = rr.z + pos*(-Rz.x - Rz.y + Rz.z);
    p->rr_s[3].x = rr.x + pos*(-Rx.x + Rx.y - Rx.z);
    p->rr_s[3].y = rr.y + pos*(-Ry.x + Ry.y - Ry.z);
    p->rr_s[3].z = rr.z + pos*(-Rz.x + Rz.y - Rz.z);
  }
}

/* rotate_vectors.cu:7-56: lab frame -> slope frame (rotation about y by the tilt). */
static inline orc_vec3 to_slope (orc_vec3 r, orc_real cost, orc_real sint)
{
  orc_vec3 q;
  q.x = r.x*cost - r.z*sint;
  q.y = r.y;
  q.z = r.x*sint + r.z*cost;
  return q;
}

void orc_rotate_vectors (orc_particle *pp, const orc_system_par *sys)
{
  long ii, n = sys->npart;
  ORC_PARALLEL_FOR
  for (ii = 0; ii < n; ii++)
  {
    int s;
    pp[ii].rrot = to_slope (pp[ii].rr, sys->cost, sys->sint);
    for (s = 0; s < 4; s++)
      pp[ii].rrot_s[s] = to_slope (pp[ii].rr_s[s], sys->cost, sys->sint);
  }
}

/* clear_forces.cu:8-29 */
void orc_clear_forces (const orc_system_par *sys, orc_vec3 *force, orc_vec3 *torque)
{
  memset (force, 0, (size_t) sys->npart*sizeof (orc_vec3));
  memset (torque, 0, (size_t) sys->npart*sizeof (orc_vec3));
}

/* get_accel.cu:9-78 */
void orc_get_accel (const orc_vec3 *force, const orc_vec3 *torque, orc_vec3 *accel,
                    orc_vec3 *ang_acc, const orc_system_par *sys, const orc_particle *pp)
{
  long ii, n = sys->npart;
  ORC_PARALLEL_FOR
  for (ii = 0; ii < n; ii++)
  {
    const orc_particle *p = &pp[ii];
    orc_vec3 I, v, w, Rx, Ry, Rz, f, t, a, wb, tb, ab, al;
    orc_real   m, rad, Cxy, Cyz, Czx, adrag, vmag;

    if (removed (sys, p->rr.x))
      continue;
    m = p->mass;  rad = p->radius;  I = p->moment_of_inertia;
    v = p->vv;  w = p->ww;  Rx = p->Rmatx;  Ry = p->Rmaty;  Rz = p->Rmatz;

    Cxy = (I.x - I.y)/I.z;
    Cyz = (I.y - I.z)/I.x;
    Czx = (I.z - I.x)/I.y;
    f = force[ii];
    t = torque[ii];

    /* Translational: F/m minus quadratic air drag, minus gravity (get_accel.cu:47-53). */
    adrag  = ORC_DRAG*rad*rad/m;
    vmag   = sqrt (v.x*v.x + v.y*v.y + v.z*v.z);
    adrag *= vmag;
    a.x = f.x/m - adrag*v.x;
    a.y = f.y/m - adrag*v.y;
    a.z = f.z/m - adrag*v.z - ORC_GRAV;

    /* Euler's equations in the body frame (get_accel.cu:56-71). */
    wb.x = w.x*Rx.x + w.y*Ry.x + w.z*Rz.x;
    wb.y = w.x*Rx.y + w.y*Ry.y + w.z*Rz.y;
    wb.z = w.x*Rx.z + w.y*Ry.z + w.z*Rz.z;
    tb.x = t.x*Rx.x + t.y*Ry.x + t.z*Rz.x;
    tb.y = t.x*Rx.y + t.y*Ry.y + t.z*Rz.y;
    tb.z = t.x*Rx.z + t.y*Ry.z + t.z*Rz.z;
    ab.x = tb.x/I.x + Cyz*wb.y*wb.z;
    ab.y = tb.y/I.y + Czx*wb.z*wb.x;
    ab.z = tb.z/I.z + Cxy*wb.x*wb.y;
    al.x = ab.x*Rx.x + ab.y*Rx.y + ab.z*Rx.z;
    al.y = ab.x*Ry.x + ab.y*Ry.y + ab.z*Ry.z;
    al.z = ab.x*Rz.x + ab.y*Rz.y + ab.z*Rz.z;

    accel[ii]   = a;
    ang_acc[ii] = al;
  }
}

/* finish_Verlet.cu:10-56 */
void orc_finish_verlet (const orc_vec3 *accel_i, const orc_vec3 *ang_acc_i, const orc_vec3 *accel_f,
                        const orc_vec3 *ang_acc_f, const orc_system_par *sys, orc_particle *pp)
{
  long ii, n = sys->npart;
  const orc_real hdt = sys->hdt;
  ORC_PARALLEL_FOR
  for (ii = 0; ii < n; ii++)
  {
    orc_particle *p = &pp[ii];
    if (removed (sys, p->rr.x))
    {
      p->vv.x = p->vv.y = p->vv.z = 0.0;
      continue;
    }
    p->vv.x += hdt*(accel_f[ii].x - accel_i[ii].x);
    p->vv.y += hdt*(accel_f[ii].y - accel_i[ii].y);
    p->vv.z += hdt*(accel_f[ii].z - accel_i[ii].z);
    p->ww.x += hdt*(ang_acc_f[ii].x - ang_acc_i[ii].x);
    p->ww.y += hdt*(ang_acc_f[ii].y - ang_acc_i[ii].y);
    p->ww.z += hdt*(ang_acc_f[ii].z - ang_acc_i[ii].z);
  }
}

/* ================================ cell list ============================== */

/* cells.cu:11-22 */
void orc_clear_cell (const orc_cell_par *cc, long *cell_vec)
{
  long ii;
  for (ii = 0; ii < cc->ntot; ii++)
    cell_vec[ii] = -1;
}

/* cells.cu:26-36 */
void orc_clear_ocup (const orc_cell_par *cc, int *nocup_vec)
{
  memset (nocup_vec, 0, (size_t) cc->ncell3*sizeof (int));
}

/* Cell coordinate of one axis as binned by cells.cu:69-77 (multiplication by cs_inv). */
static inline long bin_axis (orc_real x, orc_real xmin, orc_real inv, long n)
{
  long i = (long) (inv*(x - xmin));
  if (i == n)
    i--;
  return i;
}

/* cells.cu:40-111.  Clumps go into their cell in ascending id order; the reference's exit(1)
   cases become status codes.  An index at or beyond ncell (which the reference writes out of
   bounds) is reported as ORC_ERR_GRID_ESCAPE. */
int orc_cell_locate (const orc_cell_par *cc, const orc_system_par *sys, const orc_particle *pp,
                     int *nocup_vec, long *cell_vec)
{
  long mm;
  for (mm = 0; mm < sys->npart; mm++)
  {
    orc_vec3 r = pp[mm].rr;
    long i, j, k, idx;
    int  shift;
    if (removed (sys, r.x))
      continue;
    i = bin_axis (r.x, cc->rr_min.x, cc->cs_inv.x, cc->ncell.x);
    j = bin_axis (r.y, cc->rr_min.y, cc->cs_inv.y, cc->ncell.y);
    k = bin_axis (r.z, cc->rr_min.z, cc->cs_inv.z, cc->ncell.z);
    if (i < 0 || j < 0 || k < 0)
      return ORC_ERR_NEGATIVE_CELL;
    if (i >= cc->ncell.x || j >= cc->ncell.y || k >= cc->ncell.z)
      return ORC_ERR_GRID_ESCAPE;
    idx   = i + cc->ncell.x*(j + k*cc->ncell.y);
    shift = nocup_vec[idx];
    if (shift == cc->ntags - 1)
      return ORC_ERR_CELL_CAPACITY;
    nocup_vec[idx]++;
    cell_vec[idx*cc->ntags + (long) shift] = mm;
  }
  return ORC_OK;
}

/* cell_dim.cu:7-67: bounding box of clump centres, padded by 1.05 of the clump gyration radius
   and by a 2000-step look-ahead in +x (max vx) and -z (min vz). */
void orc_cell_dim (orc_vec3 *rr_max, orc_vec3 *rr_min, const orc_particle *pp,
                   const orc_system_par *sys)
{
  int      ii, n = (int) sys->npart;
  orc_real   rgyr = 0.5*sys->gyr_max, ddt = 2000.0*sys->dt, vxmax, vzmin;
  orc_vec3 hi, lo;

  hi = lo = pp[0].rr;
  vxmax = pp[0].vv.x;
  vzmin = pp[0].vv.z;
  for (ii = 1; ii < n; ii++)
  {
    orc_vec3 r = pp[ii].rr, v = pp[ii].vv;
    if (r.x < lo.x) lo.x = r.x;
    if (r.x > hi.x) hi.x = r.x;
    if (r.y < lo.y) lo.y = r.y;
    if (r.y > hi.y) hi.y = r.y;
    if (r.z < lo.z) lo.z = r.z;
    if (r.z > hi.z) hi.z = r.z;
    if (v.x > vxmax) vxmax = v.x;
    if (v.z < vzmin) vzmin = v.z;
  }
  hi.x += 1.05*rgyr + vxmax*ddt;
  lo.x -= 1.05*rgyr;
  hi.y += 1.05*rgyr;
  lo.y -= 1.05*rgyr;
  hi.z += 1.05*rgyr;
  lo.z -= 1.05*rgyr - vzmin*ddt;
  *rr_max = hi;
  *rr_min = lo;
}

/* avalanche_hst.cu:314-333 with the cell pitch factor of :115 (`GYR + 0.05f`, a float literal). */
void orc_grid_from_bbox (orc_cell_par *cc, const orc_system_par *sys)
{
  const orc_real dist = ORC_GYR + 0.05f;
  cc->length.x = cc->rr_max.x - cc->rr_min.x;
  cc->length.y = cc->rr_max.y - cc->rr_min.y;
  cc->length.z = cc->rr_max.z - cc->rr_min.z;
  cc->ncell.x  = (long) (cc->length.x/(dist*sys->rmax));
  cc->ncell.y  = (long) (cc->length.y/(dist*sys->rmax));
  cc->ncell.z  = (long) (cc->length.z/(dist*sys->rmax));
  cc->cell_side.x = cc->length.x/((orc_real) cc->ncell.x);
  cc->cell_side.y = cc->length.y/((orc_real) cc->ncell.y);
  cc->cell_side.z = cc->length.z/((orc_real) cc->ncell.z);
  cc->cs_inv.x = 1.0/cc->cell_side.x;
  cc->cs_inv.y = 1.0/cc->cell_side.y;
  cc->cs_inv.z = 1.0/cc->cell_side.z;
  cc->ncell3   = cc->ncell.x*cc->ncell.y*cc->ncell.z;
  cc->ntot     = cc->ncell3*cc->ntags;
}

/* ========================== particle-particle contacts ==================== */

/* Search-centre cell of force_part.cu:77-85 (division by cell_side, not multiplication). */
static inline long search_axis (orc_real x, orc_real xmin, orc_real side, long n)
{
  long i = (long) ((x - xmin)/side);
  if (i == n)
    i--;
  return i;
}

/* Visit the 27 neighbour cells of clump ll in the reference's order and call `body` for every
   other clump found (force_part.cu:88-110).  The body is the variadic tail. */
#define ORC_FOR_NEIGHBOURS(cell, cell_vec, nocup_vec, rrl, ll, mm, ...)                           \
  do {                                                                                          \
    long ci_ = search_axis ((rrl).x, (cell)->rr_min.x, (cell)->cell_side.x, (cell)->ncell.x);    \
    long cj_ = search_axis ((rrl).y, (cell)->rr_min.y, (cell)->cell_side.y, (cell)->ncell.y);    \
    long ck_ = search_axis ((rrl).z, (cell)->rr_min.z, (cell)->cell_side.z, (cell)->ncell.z);    \
    int  di_, dj_, dk_;                                                                         \
    for (di_ = -1; di_ <= 1; di_++)                                                             \
    for (dj_ = -1; dj_ <= 1; dj_++)                                                             \
    for (dk_ = -1; dk_ <= 1; dk_++)                                                             \
    {                                                                                           \
      long in_ = ci_ + di_, jn_ = cj_ + dj_, kn_ = ck_ + dk_, c_, t_, t0_, t1_;                  \
      if (in_ < 0 || jn_ < 0 || kn_ < 0 || in_ >= (cell)->ncell.x || jn_ >= (cell)->ncell.y ||  \
          kn_ >= (cell)->ncell.z)                                                               \
        continue;                                                                               \
      c_  = in_ + (cell)->ncell.x*(jn_ + (cell)->ncell.y*kn_);                                  \
      t0_ = c_*(cell)->ntags;                                                                   \
      t1_ = t0_ + (nocup_vec)[c_];                                                              \
      for (t_ = t0_; t_ < t1_; t_++)                                                            \
      {                                                                                         \
        long mm = (cell_vec)[t_];                                                               \
        if (mm == (ll))                                                                         \
          continue;                                                                             \
        __VA_ARGS__                                                                             \
      }                                                                                         \
    }                                                                                           \
  } while (0)

/* Staged sphere-sphere overlap test of force_part.cu:140-157.  Returns 1 on overlap and leaves
   the separation vector in *d and its squared norm in *dist2. */
static inline int sphere_overlap (orc_vec3 s1, orc_vec3 s2, orc_real sep2, orc_vec3 *d, orc_real *dist2)
{
  orc_real q;
  d->x = s2.x - s1.x;
  q = d->x*d->x;
  if (!(q < sep2)) return 0;
  d->y = s2.y - s1.y;
  q += d->y*d->y;
  if (!(q < sep2)) return 0;
  d->z = s2.z - s1.z;
  q += d->z*d->z;
  if (!(q < sep2)) return 0;
  *dist2 = q;
  return 1;
}

/* force_part.cu:11-266 (variant HST) and :270-531 (variant DEV: `|| xi == 0` Coulomb clause).
   Sphere (sph_id-1)%4 of clump ll against sphere (sph_id-1)/4 of every neighbour mm. */
void orc_force_part (orc_vec3 *force, orc_vec3 *torque, const long *cell_vec, const int *nocup_vec,
                     const orc_particle *pp, const orc_system_par *sys, const orc_cell_par *cell,
                     int sph_id, int variant)
{
  const int    sl = (sph_id - 1)%4, sm = (sph_id - 1)/4;
  const orc_real mu = sys->mu_pp, kappa = sys->kappa_pp, gamma = sys->gamma_pp, dt = sys->dt;
  const orc_real cns_1 = sys->fr_fact_pp;
  long ll;

  ORC_PARALLEL_FOR
  for (ll = 0; ll < sys->npart; ll++)
  {
    const orc_particle *pl = &pp[ll];
    orc_vec3 rrl = pl->rr, vvl, wwl, s1, ff, tq;
    orc_real   rad_1, massl;

    if (removed (sys, rrl.x))
      continue;
    vvl = pl->vv;  wwl = pl->ww;  rad_1 = pl->radius;
    ff = force[ll];  tq = torque[ll];
    massl = ORC_SPH_FACT*pl->density*rad_1*rad_1*rad_1;
    s1 = pl->rr_s[sl];

    ORC_FOR_NEIGHBOURS (cell, cell_vec, nocup_vec, rrl, ll, mm, {
      const orc_particle *pm = &pp[mm];
      orc_real   rad_2 = pm->radius, massm, meff, km, gm, sep, sep2, dist2, dist;
      orc_vec3 d, nv, rrc, vl, vm, dvvc, fs;

      massm = ORC_SPH_FACT*pm->density*rad_2*rad_2*rad_2;
      meff  = 0.5*(massm + massl);
      km    = 0.5*kappa*meff;
      gm    = 0.5*gamma*meff;
      sep   = rad_1 + rad_2;
      sep2  = sep*sep;
      if (sphere_overlap (s1, pm->rr_s[sm], sep2, &d, &dist2))
      {
        dist  = sqrt (dist2);
        nv.x  = d.x/dist;
        nv.y  = d.y/dist;
        nv.z  = d.z/dist;
        rrc.x = s1.x + rad_1*nv.x;
        rrc.y = s1.y + rad_1*nv.y;
        rrc.z = s1.z + rad_1*nv.z;
        vl = point_velocity (vvl, wwl, rrc, rrl);
        vm = point_velocity (pm->vv, pm->ww, rrc, pm->rr);
        dvvc.x = vm.x - vl.x;
        dvvc.y = vm.y - vl.y;
        dvvc.z = vm.z - vl.z;
        if (contact_law (dvvc, nv, sep - dist, km, gm, massl, mu, cns_1, dt,
                         variant == ORC_FRICTION_DEV, 0, &fs))
          accumulate (&ff, &tq, fs, rrc, rrl);
      }
    });

    force[ll]  = ff;
    torque[ll] = tq;
  }
}

long orc_contact_pairs (long *out, long cap, const long *cell_vec, const int *nocup_vec,
                        const orc_particle *pp, const orc_system_par *sys, const orc_cell_par *cell,
                        int active)
{
  const orc_real mu = sys->mu_pp, kappa = sys->kappa_pp, gamma = sys->gamma_pp, dt = sys->dt;
  const orc_real cns_1 = sys->fr_fact_pp;
  long count = 0, ll;
  int  sph_id;

  for (sph_id = 1; sph_id <= 16; sph_id++)
  for (ll = 0; ll < sys->npart; ll++)
  {
    const orc_particle *pl = &pp[ll];
    const int sl = (sph_id - 1)%4, sm = (sph_id - 1)/4;
    orc_vec3 rrl = pl->rr;
    orc_real   rad_1 = pl->radius, massl;
    if (removed (sys, rrl.x))
      continue;
    massl = ORC_SPH_FACT*pl->density*rad_1*rad_1*rad_1;
    ORC_FOR_NEIGHBOURS (cell, cell_vec, nocup_vec, rrl, ll, mm, {
      const orc_particle *pm = &pp[mm];
      orc_real   rad_2 = pm->radius, sep = rad_1 + rad_2, dist2;
      orc_vec3 d;
      if (sphere_overlap (pl->rr_s[sl], pm->rr_s[sm], sep*sep, &d, &dist2))
      {
        int keep = 1;
        if (active)
        {
          orc_real   massm = ORC_SPH_FACT*pm->density*rad_2*rad_2*rad_2, meff = 0.5*(massm + massl);
          orc_real   dist = sqrt (dist2);
          orc_vec3 nv, rrc, vl, vm, dvvc, fs;
          nv.x = d.x/dist;  nv.y = d.y/dist;  nv.z = d.z/dist;
          rrc.x = pl->rr_s[sl].x + rad_1*nv.x;
          rrc.y = pl->rr_s[sl].y + rad_1*nv.y;
          rrc.z = pl->rr_s[sl].z + rad_1*nv.z;
          vl = point_velocity (pl->vv, pl->ww, rrc, rrl);
          vm = point_velocity (pm->vv, pm->ww, rrc, pm->rr);
          dvvc.x = vm.x - vl.x;  dvvc.y = vm.y - vl.y;  dvvc.z = vm.z - vl.z;
          keep = contact_law (dvvc, nv, sep - dist, 0.5*kappa*meff, 0.5*gamma*meff, massl, mu,
                              cns_1, dt, 0, 0, &fs);
        }
        if (keep)
        {
          if (count < cap)
          {
            out[3*count]     = ll;
            out[3*count + 1] = mm;
            out[3*count + 2] = sph_id;
          }
          count++;
        }
      }
    });
  }
  return count;
}

/* ================================ boundaries ============================== */

/* Mass of one sphere in the wall routines' operand order (force_walls.cu:47). */
static inline orc_real wall_sphere_mass (const orc_particle *p)
{
  orc_real ri = p->radius;
  return ORC_SPH_FACT*ri*ri*ri*p->density;
}

/* force_hop.cu:9-244.  nw = 0: rear/front (x = 0 / 15), 1: left/right (y = 7.5 / 22.5),
   2: bottom door (z = 25, only while time < 0).  Only spheres with z >= 25 and x <= 15. */
void orc_force_hop (orc_vec3 *force, orc_vec3 *torque, const orc_system_par *sys,
                    const orc_particle *pp, int nw)
{
  const orc_real mu = sys->mu_pw, kappa = sys->kappa_pw, gamma = sys->gamma_pw, dt = sys->dt;
  const orc_real cns_1 = sys->fr_fact_pw, time = sys->time;
  long ii;

  ORC_PARALLEL_FOR
  for (ii = 0; ii < sys->npart; ii++)
  {
    const orc_particle *p = &pp[ii];
    orc_vec3 ff = force[ii], tq = torque[ii];
    orc_real   ri = p->radius, mass = wall_sphere_mass (p), km = 0.5*kappa*mass, gm = 0.5*gamma*mass;
    int      ns;

    for (ns = 0; ns < 4; ns++)
    {
      orc_vec3 s = p->rr_s[ns], rrc, nv;
      orc_real   dist, comp = 0.0;
      int      touch = 0;
      if (s.z < ORC_HOP_HEIGHT || s.x > ORC_HOP_WIDTH)
        continue;
      if (nw == 0)
      {
        dist = s.x - 0.0;
        if (dist <= ri)
        {
          touch = 1;  rrc.x = 0.0;  rrc.y = s.y;  rrc.z = s.z;
          nv.x = -1.0;  nv.y = 0.0;  nv.z = 0.0;  comp = ri - dist;
        }
        dist = ORC_HOP_WIDTH - s.x;
        if (dist <= ri)
        {
          touch = 2;  rrc.x = ORC_HOP_WIDTH;  rrc.y = s.y;  rrc.z = s.z;
          nv.x = 1.0;  nv.y = 0.0;  nv.z = 0.0;  comp = ri - dist;
        }
      }
      else if (nw == 1)
      {
        dist = s.y - ORC_YHOP_L;
        if (dist <= ri)
        {
          touch = 3;  rrc.x = s.x;  rrc.y = ORC_YHOP_L;  rrc.z = s.z;
          nv.x = 0.0;  nv.y = -1.0;  nv.z = 0.0;  comp = ri - dist;
        }
        dist = ORC_YHOP_R - s.y;
        if (dist <= ri)
        {
          touch = 4;  rrc.x = s.x;  rrc.y = ORC_YHOP_R;  rrc.z = s.z;
          nv.x = 0.0;  nv.y = 1.0;  nv.z = 0.0;  comp = ri - dist;
        }
      }
      else if (nw == 2)
      {
        dist = s.z - ORC_HOP_HEIGHT;
        if (dist <= ri)
        {
          touch = time < 0.0 ? 5 : 0;   /* the door is open once time >= 0 */
          rrc.x = s.x;  rrc.y = s.y;  rrc.z = ORC_HOP_HEIGHT;
          nv.x = 0.0;  nv.y = 0.0;  nv.z = -1.0;  comp = ri - dist;
        }
      }
      if (touch)
        wall_contact (p, rrc, nv, comp, km, gm, mass, mu, cns_1, dt, 0, &ff, &tq);
    }
    force[ii]  = ff;
    torque[ii] = tq;
  }
}

/* Slope frame -> lab frame (force_funnel.cu:88-93). */
static inline orc_vec3 to_lab (orc_vec3 q, orc_real cost, orc_real sint)
{
  orc_vec3 r;
  r.x = q.x*cost + q.z*sint;
  r.y = q.y;
  r.z = q.z*cost - q.x*sint;
  return r;
}

/* force_funnel.cu:9-213: two converging planar walls of the funnel, in the slope frame. */
void orc_force_funnel (orc_vec3 *force, orc_vec3 *torque, const orc_system_par *sys,
                       const orc_particle *pp, const orc_funnel *fun)
{
  const orc_real mu = sys->mu_pw, kappa = sys->kappa_pw, gamma = sys->gamma_pw, dt = sys->dt;
  const orc_real cns_1 = sys->fr_fact_pw, cost = sys->cost, sint = sys->sint;
  const orc_real sinfi = fun->sinfi, cosfi = fun->cosfi, tanfi = fun->tanfi;
  long ii;

  ORC_PARALLEL_FOR
  for (ii = 0; ii < sys->npart; ii++)
  {
    const orc_particle *p = &pp[ii];
    orc_vec3 ff = force[ii], tq = torque[ii];
    orc_real   ri = p->radius, mass = wall_sphere_mass (p), km = 0.5*kappa*mass, gm = 0.5*gamma*mass;
    int      ns;

    for (ns = 0; ns < 4; ns++)
    {
      orc_vec3 q = p->rrot_s[ns], qc, nr, rrc, nv;
      orc_real   dist, comp = 0.0;
      int      touch = 0;
      if (q.x > ORC_LFUNNEL - ri*sinfi)
        continue;
      dist = fabs (q.y - q.x*tanfi)*cosfi;
      if (dist <= ri)
      {
        touch = 1;
        qc.x = q.x + dist*sinfi;  qc.y = q.y - dist*cosfi;  qc.z = q.z;
        nr.x = sinfi;  nr.y = -cosfi;  nr.z = 0.0;
        rrc = to_lab (qc, cost, sint);
        nv  = to_lab (nr, cost, sint);
        comp = ri - dist;
      }
      dist = fabs (ORC_YFUNNEL - q.y - q.x*tanfi)*cosfi;
      if (dist <= ri)
      {
        touch = 2;
        qc.x = q.x + dist*sinfi;  qc.y = q.y + dist*cosfi;  qc.z = q.z;
        nr.x = sinfi;  nr.y = cosfi;  nr.z = 0.0;
        rrc = to_lab (qc, cost, sint);
        nv  = to_lab (nr, cost, sint);
        comp = ri - dist;
      }
      if (touch)
        wall_contact (p, rrc, nv, comp, km, gm, mass, mu, cns_1, dt, 0, &ff, &tq);
    }
    force[ii]  = ff;
    torque[ii] = tq;
  }
}

/* force_funnel.cu:216-404: edge contact with the two vertical corner lines at x_rot = LFUNNEL. */
void orc_force_fcorners (orc_vec3 *force, orc_vec3 *torque, const orc_system_par *sys,
                         const orc_funnel *fun, const orc_particle *pp)
{
  const orc_real mu = sys->mu_pw, kappa = sys->kappa_pw, gamma = sys->gamma_pw, dt = sys->dt;
  const orc_real cns_1 = sys->fr_fact_pw, sin_fa = fun->sinfi, cost = sys->cost, sint = sys->sint;
  const orc_real yfun_l = sys->dy2, yfun_r = sys->side.y + sys->dy2, hsy = sys->dy2 + sys->side.y/2.0;
  long ii;

  ORC_PARALLEL_FOR
  for (ii = 0; ii < sys->npart; ii++)
  {
    const orc_particle *p = &pp[ii];
    orc_vec3 ff = force[ii], tq = torque[ii];
    orc_real   ri = p->radius, mass = wall_sphere_mass (p), km = 0.5*kappa*mass, gm = 0.5*gamma*mass;
    int      ns;

    for (ns = 0; ns < 4; ns++)
    {
      orc_vec3 q = p->rrot_s[ns], d, nr, qc;
      orc_real   yc, sep2, dist2, dist;
      if (q.x < ORC_LFUNNEL - ri*sin_fa || q.x > ORC_LFUNNEL + ri)
        continue;
      if (q.y > yfun_r || q.y < yfun_l)
        continue;
      yc   = (q.y <= hsy) ? yfun_l : yfun_r;
      sep2 = ri*ri;
      d.x  = ORC_LFUNNEL - q.x;
      dist2 = d.x*d.x;
      if (dist2 > sep2)
        continue;
      d.y = yc - q.y;
      dist2 += d.y*d.y;
      if (dist2 > sep2)
        continue;
      dist = sqrt (dist2);
      nr.x = d.x/dist;  nr.y = d.y/dist;  nr.z = 0.0;
      qc.x = q.x + ri*nr.x;  qc.y = q.y + ri*nr.y;  qc.z = q.z;
      wall_contact (p, to_lab (qc, cost, sint), to_lab (nr, cost, sint), ri - dist, km, gm, mass,
                    mu, cns_1, dt, 1, &ff, &tq);
    }
    force[ii]  = ff;
    torque[ii] = tq;
  }
}

/* force_walls.cu:9-199: flume side walls y = dy2 and y = side.y + dy2 beyond the funnel. */
void orc_force_walls (orc_vec3 *force, orc_vec3 *torque, const orc_system_par *sys,
                      const orc_particle *pp)
{
  const orc_real mu = sys->mu_pw, kappa = sys->kappa_pw, gamma = sys->gamma_pw, dt = sys->dt;
  const orc_real cns_1 = sys->fr_fact_pw, yleft = sys->dy2, yright = sys->side.y + sys->dy2;
  long ii;

  ORC_PARALLEL_FOR
  for (ii = 0; ii < sys->npart; ii++)
  {
    const orc_particle *p = &pp[ii];
    orc_vec3 ff, tq;
    orc_real   ri, mass, km, gm;
    int      ns;

    if (removed (sys, p->rr.x))
      continue;
    ff = force[ii];  tq = torque[ii];
    ri = p->radius;  mass = wall_sphere_mass (p);  km = 0.5*kappa*mass;  gm = 0.5*gamma*mass;
    for (ns = 0; ns < 4; ns++)
    {
      orc_vec3 s = p->rr_s[ns], rrc, nv;
      orc_real   dist, comp = 0.0;
      int      touch = 0;
      if (p->rrot_s[ns].x <= ORC_LFUNNEL)
        continue;
      dist = s.y - yleft;
      if (dist <= ri)
      {
        touch = 1;  rrc.x = s.x;  rrc.y = yleft;  rrc.z = s.z;
        nv.x = 0.0;  nv.y = -1.0;  nv.z = 0.0;  comp = ri - dist;
      }
      dist = yright - s.y;
      if (dist <= ri)
      {
        touch = 2;  rrc.x = s.x;  rrc.y = yright;  rrc.z = s.z;
        nv.x = 0.0;  nv.y = 1.0;  nv.z = 0.0;  comp = ri - dist;
      }
      if (touch)
        wall_contact (p, rrc, nv, comp, km, gm, mass, mu, cns_1, dt, 0, &ff, &tq);
    }
    force[ii]  = ff;
    torque[ii] = tq;
  }
}

/* force_flume.cu:10-182: the inclined bed z = -tan(tilt) x. */
void orc_force_flume (orc_vec3 *force, orc_vec3 *torque, const orc_system_par *sys,
                      const orc_particle *pp)
{
  const orc_real mu = sys->mu_pw, kappa = sys->kappa_pw, gamma = sys->gamma_pw, dt = sys->dt;
  const orc_real cns_1 = sys->fr_fact_pw, sint = sys->sint, cost = sys->cost, tant = sint/cost;
  long ii;

  ORC_PARALLEL_FOR
  for (ii = 0; ii < sys->npart; ii++)
  {
    const orc_particle *p = &pp[ii];
    orc_vec3 ff, tq, nv;
    orc_real   ri, mass, km, gm;
    int      ns;

    if (removed (sys, p->rr.x))
      continue;
    ff = force[ii];  tq = torque[ii];
    ri = p->radius;  mass = wall_sphere_mass (p);  km = 0.5*kappa*mass;  gm = 0.5*gamma*mass;
    nv.x = -sint;  nv.y = 0.0;  nv.z = -cost;
    for (ns = 0; ns < 4; ns++)
    {
      orc_vec3 s = p->rr_s[ns], rrc;
      orc_real   rect = -tant*s.x - s.z, dist = fabs (cost*rect);
      if (dist <= ri)
      {
        rrc.x = s.x - dist*sint;
        rrc.y = s.y;
        rrc.z = s.z - dist*cost;
        wall_contact (p, rrc, nv, ri - dist, km, gm, mass, mu, cns_1, dt, 0, &ff, &tq);
      }
    }
    force[ii]  = ff;
    torque[ii] = tq;
  }
}

/* ================================ drivers ================================ */

int orc_forces (const orc_system_par *sys, const orc_funnel *fun, const orc_cell_par *cell,
                orc_particle *pp, orc_work *w, int phase, int variant)
{
  int st, s;
  if (cell->ntot > w->cell_vec_cap || cell->ncell3 > w->nocup_cap)
    return ORC_ERR_GRID_ESCAPE;
  orc_clear_forces (sys, w->force, w->torque);
  orc_clear_cell (cell, w->cell_vec);
  orc_clear_ocup (cell, w->nocup_vec);
  st = orc_cell_locate (cell, sys, pp, w->nocup_vec, w->cell_vec);
  if (st != ORC_OK)
    return st;
  if (phase == 0)
  {
    /* Hopper fill: particles, then the three hopper wall groups (avalanche_hst.cu:455-461). */
    for (s = 1; s <= 16; s++)
      orc_force_part (w->force, w->torque, w->cell_vec, w->nocup_vec, pp, sys, cell, s, variant);
    for (s = 0; s < 3; s++)
      orc_force_hop (w->force, w->torque, sys, pp, s);
  }
  else
  {
    /* Avalanche: hop x3, funnel, corners, side walls, particles, bed (avalanche_hst.cu:688-704). */
    for (s = 0; s < 3; s++)
      orc_force_hop (w->force, w->torque, sys, pp, s);
    orc_force_funnel (w->force, w->torque, sys, pp, fun);
    orc_force_fcorners (w->force, w->torque, sys, fun, pp);
    orc_force_walls (w->force, w->torque, sys, pp);
    for (s = 1; s <= 16; s++)
      orc_force_part (w->force, w->torque, w->cell_vec, w->nocup_vec, pp, sys, cell, s, variant);
    orc_force_flume (w->force, w->torque, sys, pp);
  }
  orc_get_accel (w->force, w->torque, w->acc_f, w->anga_f, sys, pp);
  return ORC_OK;
}

int orc_step (orc_system_par *sys, const orc_funnel *fun, const orc_cell_par *cell,
              orc_particle *pp, orc_work *w, int phase, int variant)
{
  int st;
  orc_vec3 *tmp;
  orc_init_verlet (w->acc_i, w->anga_i, sys, pp);
  sys->time += sys->dt;
  if (phase != 0)
    orc_rotate_vectors (pp, sys);
  st = orc_forces (sys, fun, cell, pp, w, phase, variant);
  if (st != ORC_OK)
    return st;
  orc_finish_verlet (w->acc_i, w->anga_i, w->acc_f, w->anga_f, sys, pp);
  tmp = w->acc_i;  w->acc_i  = w->acc_f;  w->acc_f  = tmp;
  tmp = w->anga_i; w->anga_i = w->anga_f; w->anga_f = tmp;
  return ORC_OK;
}
