/*
 * ref_shim.cu -- C-linkage wrappers around the reference's own host routines.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/build.py compiles this file together with
 * the reference's unmodified sources, read where they lie in the reference
 * tree (include path -I<reference>), into oracle/_ref/libaf3d_ref.so.  The
 * tests use it to pin the oracle restatement (oracle/af3d_oracle.c) and to
 * generate tests/golden/.  Structs passed by value in the reference are
 * passed by pointer here so that ctypes can call them.
 */
#include "cabecera.hu"

extern "C" {

void ref_init_Verlet_hst (double3 *a, double3 *al, const system_par *s, particle *pp)
{ init_Verlet_hst (a, al, *s, pp); }

void ref_rotate_vectors_hst (particle *pp, const system_par *s)
{ rotate_vectors_hst (pp, *s); }

void ref_clear_forces_hst (const system_par *s, double3 *f, double3 *t)
{ clear_forces_hst (*s, f, t); }

void ref_clear_cell_hst (const cell_par *c, long *cv)
{ clear_cell_hst (*c, cv); }

void ref_clear_ocup_hst (const cell_par *c, int *no)
{ clear_ocup_hst (*c, no); }

void ref_cell_locate_hst (const cell_par *c, const system_par *s, particle *pp, int *no, long *cv)
{ cell_locate_hst (*c, *s, pp, no, cv); }

void ref_force_hop_hst (double3 *f, double3 *t, const system_par *s, particle *pp, int nw)
{ force_hop_hst (f, t, *s, pp, (char) nw); }

void ref_force_funnel_hst (double3 *f, double3 *t, const system_par *s, particle *pp, const Funnel *fu)
{ force_funnel_hst (f, t, *s, pp, *fu); }

void ref_force_fcorners_hst (double3 *f, double3 *t, const system_par *s, const Funnel *fu, particle *pp)
{ force_fcorners_hst (f, t, *s, *fu, pp); }

void ref_force_walls_hst (double3 *f, double3 *t, const system_par *s, particle *pp)
{ force_walls_hst (f, t, *s, pp); }

void ref_force_part_hst (double3 *f, double3 *t, long *cv, int *no, particle *pp, const system_par *s,
                         const cell_par *c, int sph_id)
{ force_part_hst (f, t, cv, no, pp, *s, *c, sph_id); }

void ref_force_flume_hst (double3 *f, double3 *t, const system_par *s, particle *pp)
{ force_flume_hst (f, t, *s, pp); }

void ref_get_accel_hst (double3 *f, double3 *t, double3 *a, double3 *al, const system_par *s, particle *pp)
{ get_accel_hst (f, t, a, al, *s, pp); }

void ref_finish_Verlet_hst (double3 *ai, double3 *ali, double3 *af, double3 *alf, const system_par *s,
                            particle *pp)
{ finish_Verlet_hst (ai, ali, af, alf, *s, pp); }

void ref_cell_dim (double3 *rmax, double3 *rmin, particle *pp, const system_par *s)
{ cell_dim (rmax, rmin, pp, *s); }

int ref_error_check (const system_par *s, char *msg)
{ return error_check (*s, msg); }

void ref_generate_particles (particle *pp, const system_par *s)
{ generate_particles (pp, *s); }

void ref_calculate_particle_parameters_hst (const system_par *s, particle *pp)
{ calculate_particle_parameters_hst (*s, pp); }

void ref_place_particles (const system_par *s, particle *pp)
{ place_particles (*s, pp); }

void ref_set_initial_velocity (const system_par *s, particle *pp)
{ set_initial_velocity (*s, pp); }

double ref_rannew64 (long *idum)
{ return RAN (idum); }

long ref_sizeof_particle (void)   { return (long) sizeof (particle); }
long ref_sizeof_system_par (void) { return (long) sizeof (system_par); }
long ref_sizeof_cell_par (void)   { return (long) sizeof (cell_par); }

}
