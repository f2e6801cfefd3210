/*
 * af3d_oracle.h -- CPU oracle for the AvalancheFlume3D clump-DEM step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * host (`*_hst`) step routines, used by the test-suite as the parity checker
 * and by bench.py as the timed CPU baseline.  The product path never links,
 * loads or calls it.
 *
 * Parity: pinned bit-exactly against the reference's own routines compiled
 * from source (oracle/build.py -> oracle/_ref/libaf3d_ref.so) by
 * tests/test_oracle_pin.py, and against the committed fixtures in
 * tests/golden/ generated from those routines.
 *
 * Every arithmetic expression keeps the reference's FP64 evaluation order,
 * and the library is compiled with -ffp-contract=off, so results are
 * bit-identical to the reference on IEEE hardware (+, -, *, /, sqrt are
 * correctly rounded; sin/cos/log come from the platform libm).
 *
 * Struct layouts are binary-identical to the reference's `system_par`,
 * `Funnel`, `particle` and `cell_par` (cabecera.hu:34-112).
 */
#ifndef AF3D_ORACLE_H
#define AF3D_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* The real type of the state and of every expression: double.  The tangent-linear model
   (af3d_tangent.cpp) compiles af3d_oracle.c a second time, as C++, with ORC_REAL set to a
   dual-number type carrying directional derivatives beside each value. */
#ifndef ORC_REAL
#define ORC_REAL double
#endif
typedef ORC_REAL orc_real;

typedef struct { orc_real x, y, z; } orc_vec3;
typedef struct { long x, y, z; } orc_lvec3;

/* cabecera.hu:34-66 (256 bytes). */
typedef struct {
  long     npart;
  orc_real   dt, hdt, rmin, rmax, v0, time, eps_pp, eps_pw, kappa_pp, kappa_pw, gamma_pp, gamma_pw,
           mu_pp, mu_pw, t_coll, tot_mass, tilt, xhopper, Lflume, gyr_max, fr_fact_pp, fr_fact_pw,
           sint, cost, sintg, costg, xfunnel, dy2;
  orc_vec3 side;
} orc_system_par;

/* cabecera.hu:69-74. */
typedef struct { orc_real sinfi, cosfi, tanfi; } orc_funnel;

/* cabecera.hu:77-98 (408 bytes).  rr_s[0..3] are rr_a..rr_d, rrot_s[0..3] are rrot_a..rrot_d. */
typedef struct {
  orc_real   radius, mass, density;
  orc_vec3 moment_of_inertia;
  orc_vec3 rr_s[4];
  orc_vec3 rrot_s[4];
  orc_vec3 rr, rrot, vv, ww, Rmatx, Rmaty, Rmatz;
} orc_particle;

/* cabecera.hu:101-112 (168 bytes). */
typedef struct {
  long      ntags, ncell3;
  orc_lvec3 ncell;
  long      ntot;
  orc_vec3  cell_side, cs_inv, rr_max, rr_min, length;
} orc_cell_par;

/* Friction variants: the host particle contact omits the `|| xi == 0` Coulomb clause
   (force_part.cu:224), the device one has it (force_part.cu:487). */
enum { ORC_FRICTION_HST = 0, ORC_FRICTION_DEV = 1 };

/* Status codes of the routines that the reference ends with exit(1). */
enum { ORC_OK = 0, ORC_ERR_NEGATIVE_CELL = 1, ORC_ERR_CELL_CAPACITY = 2, ORC_ERR_GRID_ESCAPE = 3 };

void orc_set_threads (int nthreads);

/* ---- per-routine restatements (same argument meaning as the reference) ---- */
void orc_init_verlet    (const orc_vec3 *accel, const orc_vec3 *ang_acc, const orc_system_par *sys,
                         orc_particle *pp);
void orc_rotate_vectors (orc_particle *pp, const orc_system_par *sys);
void orc_clear_forces   (const orc_system_par *sys, orc_vec3 *force, orc_vec3 *torque);
void orc_clear_cell     (const orc_cell_par *cc, long *cell_vec);
void orc_clear_ocup     (const orc_cell_par *cc, int *nocup_vec);
int  orc_cell_locate    (const orc_cell_par *cc, const orc_system_par *sys, const orc_particle *pp,
                         int *nocup_vec, long *cell_vec);
void orc_force_hop      (orc_vec3 *force, orc_vec3 *torque, const orc_system_par *sys,
                         const orc_particle *pp, int nw);
void orc_force_funnel   (orc_vec3 *force, orc_vec3 *torque, const orc_system_par *sys,
                         const orc_particle *pp, const orc_funnel *fun);
void orc_force_fcorners (orc_vec3 *force, orc_vec3 *torque, const orc_system_par *sys,
                         const orc_funnel *fun, const orc_particle *pp);
void orc_force_walls    (orc_vec3 *force, orc_vec3 *torque, const orc_system_par *sys,
                         const orc_particle *pp);
void orc_force_part     (orc_vec3 *force, orc_vec3 *torque, const long *cell_vec, const int *nocup_vec,
                         const orc_particle *pp, const orc_system_par *sys, const orc_cell_par *cell,
                         int sph_id, int variant);
void orc_force_flume    (orc_vec3 *force, orc_vec3 *torque, const orc_system_par *sys,
                         const orc_particle *pp);
void orc_get_accel      (const orc_vec3 *force, const orc_vec3 *torque, orc_vec3 *accel,
                         orc_vec3 *ang_acc, const orc_system_par *sys, const orc_particle *pp);
void orc_finish_verlet  (const orc_vec3 *accel_i, const orc_vec3 *ang_acc_i, const orc_vec3 *accel_f,
                         const orc_vec3 *ang_acc_f, const orc_system_par *sys, orc_particle *pp);

/* cell_dim.cu:7-67 plus the grid derivation of avalanche_hst.cu:314-333. */
void orc_cell_dim       (orc_vec3 *rr_max, orc_vec3 *rr_min, const orc_particle *pp,
                         const orc_system_par *sys);
void orc_grid_from_bbox (orc_cell_par *cc, const orc_system_par *sys);

/* Contact-pair enumeration with the reference's staged overlap test (force_part.cu:140-157):
   writes (ll, mm, sph_id) triples of overlapping sphere pairs in the reference's visiting order
   (sph_id, then the 27 cells in idel/jdel/kdel order, then slot order).  `active` = 1 keeps only
   pairs whose normal force is repulsive.  Returns the number of pairs (may exceed cap). */
long orc_contact_pairs  (long *out, long cap, const long *cell_vec, const int *nocup_vec,
                         const orc_particle *pp, const orc_system_par *sys, const orc_cell_par *cell,
                         int active);

/* ---- step drivers (avalanche_hst.cu:438-467 fill step, :668-710 avalanche step) ---- */
typedef struct {
  orc_vec3 *force, *torque, *acc_i, *anga_i, *acc_f, *anga_f;
  long     *cell_vec;
  int      *nocup_vec;
  long      cell_vec_cap, nocup_cap;
} orc_work;

/* One step of the avalanche (phase = 1) or hopper-fill (phase = 0) sequence, including the
   `time += dt` and the final swap of the acceleration buffers.  Returns an ORC_* status. */
int  orc_step (orc_system_par *sys, const orc_funnel *fun, const orc_cell_par *cell,
               orc_particle *pp, orc_work *w, int phase, int variant);

/* Force pass only (clear, cells, every force routine of the phase, get_accel into acc_f). */
int  orc_forces (const orc_system_par *sys, const orc_funnel *fun, const orc_cell_par *cell,
                 orc_particle *pp, orc_work *w, int phase, int variant);

#ifdef __cplusplus
}
#endif
#endif
