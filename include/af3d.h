/*
 * af3d.h -- C ABI of the GB300 clump-DEM engine (drop-in for the step loop of
 * AvalancheFlume3D).
 *
 * The reference's step loop launches one routine per call on the default
 * stream and keeps every array in caller-owned memory.  Here the state is
 * device-resident inside an opaque context: the caller imports the reference's
 * `particle` array once (host memory), calls one entry point per reference
 * routine -- or af3d_step() for K fused, graph-captured steps -- and exports
 * the state whenever it wants host copies.  Every entry point returns an
 * af3d_status; nothing calls exit().
 *
 * Structs are binary-identical to the reference's (cabecera.hu:34-112), so a
 * reference driver can pass its own `system_par`, `Funnel`, `particle` and
 * `cell_par` objects.  All arithmetic is FP64 in cgs units.
 */
#ifndef AF3D_H
#define AF3D_H

#include <stddef.h>
#include <stdint.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AF3D_ABI_VERSION 1

typedef struct { double x, y, z; } af3d_vec3;
typedef struct { long x, y, z; } af3d_lvec3;

/* system_par, cabecera.hu:34-66 (256 bytes). */
typedef struct {
  long      npart;
  double    dt, hdt, rmin, rmax, v0, time, eps_pp, eps_pw, kappa_pp, kappa_pw, gamma_pp, gamma_pw,
            mu_pp, mu_pw, t_coll, tot_mass, tilt, xhopper, Lflume, gyr_max, fr_fact_pp, fr_fact_pw,
            sint, cost, sintg, costg, xfunnel, dy2;
  af3d_vec3 side;
} af3d_system_par;

/* Funnel, cabecera.hu:69-74. */
typedef struct { double sinfi, cosfi, tanfi; } af3d_funnel;

/* particle, cabecera.hu:77-98 (408 bytes); rr_s[k] = rr_a..rr_d, rrot_s[k] = rrot_a..rrot_d. */
typedef struct {
  double    radius, mass, density;
  af3d_vec3 moment_of_inertia;
  af3d_vec3 rr_s[4];
  af3d_vec3 rrot_s[4];
  af3d_vec3 rr, rrot, vv, ww, Rmatx, Rmaty, Rmatz;
} af3d_particle;

/* cell_par, cabecera.hu:101-112 (168 bytes). */
typedef struct {
  long       ntags, ncell3;
  af3d_lvec3 ncell;
  long       ntot;
  af3d_vec3  cell_side, cs_inv, rr_max, rr_min, length;
} af3d_cell_par;

/* The 16 positional lines of DataInput.dat (avalanche_hst.cu:34-81). */
typedef struct {
  long   npart;
  double width, hopper_height, rmin, rmax, v0, dt, eps_pw, mu_pw, eps_pp, mu_pp, t_coll, Lflume,
         tilt_deg;
  long   ntags;
  int    print_flag;
} af3d_inputs;

typedef int af3d_status;
enum {
  AF3D_OK = 0,
  AF3D_ERR_ARG = 1,            /* bad argument or call order                                   */
  AF3D_ERR_CUDA = 2,           /* a CUDA runtime call failed (af3d_last_error() has the text)  */
  AF3D_ERR_NOMEM = 3,
  AF3D_ERR_GRID_ESCAPE = 4,    /* a clump left the cell grid between re-grids (reference: UB)  */
  AF3D_ERR_NEGATIVE_CELL = 5,  /* negative cell index (reference: exit(1), cells.cu:79-88)     */
  AF3D_ERR_CELL_CAPACITY = 6,  /* a cell holds >= ntags clumps (reference: exit(1), :96-102)   */
  AF3D_ERR_NAN = 7,            /* non-finite force or acceleration                             */
  AF3D_ERR_IO = 8,             /* file missing or malformed                                    */
  AF3D_ERR_INPUT = 9           /* DataInput values rejected by error_check (error_check.cu:3)  */
};

/* Friction variant of the particle-particle tangential law: the host routine omits the
   `|| xi == 0` clause of the Coulomb test (force_part.cu:224), the device one has it (:487). */
enum { AF3D_FRICTION_HST = 0, AF3D_FRICTION_DEV = 1 };

/* FP64 arithmetic of af3d_step and af3d_forces (the per-routine entry points are always exact).
   EXACT: the reference's operations in its order, no contraction: forces, torques and
   accelerations bit-identical to the reference host routines on the same input.  FAST: the same
   FP64 physics with contracted multiply-adds and reciprocal-square-root normalisation (no
   reference counterpart): forces within ~1e-14 relative of the reference, trajectories within
   1e-8 relative over 100 steps. */
enum { AF3D_FP_EXACT = 0, AF3D_FP_FAST = 1 };

/* Phase of the reference loop: hopper filling (avalanche_hst.cu:401-601) or avalanche (:618-856). */
enum { AF3D_PHASE_FILL = 0, AF3D_PHASE_AVALANCHE = 1 };
/* Objectives of af3d_adjoint (no counterpart in the reference; af3d_set_objective). */
enum { AF3D_OBJ_CENTROID = 0, AF3D_OBJ_RUNOUT = 1 };

typedef struct af3d_ctx af3d_ctx;

/* ---- context ---------------------------------------------------------------------------- */

/* Create a context for sys->npart clumps on the current CUDA device.  ntags > 0 enforces the
   reference's cell capacity (at most ntags-1 clumps per cell, cells.cu:96); ntags <= 0 lifts it.
   Replaces the cudaMalloc block of avalanche_dev.cu:140-158. */
af3d_status af3d_create (const af3d_system_par *sys, const af3d_funnel *fun, long ntags, int phase,
                         af3d_ctx **out);
af3d_status af3d_destroy (af3d_ctx *ctx);
af3d_status af3d_set_stream (af3d_ctx *ctx, void *cuda_stream);      /* cudaStream_t, 0 = own */
af3d_status af3d_set_friction (af3d_ctx *ctx, int variant);          /* AF3D_FRICTION_*       */
af3d_status af3d_set_fp_mode (af3d_ctx *ctx, int mode);              /* AF3D_FP_*, default EXACT */
const char *af3d_last_error (void);
int         af3d_abi_version (void);

/* Copy the reference particle array (host memory) and the current accelerations a_i, alpha_i
   in/out (avalanche_dev.cu:347 / :716).  acc/anga may be NULL (import: zeros; export: skipped).
   Export writes the slope-frame copies rrot from the current positions. */
af3d_status af3d_import_particles (af3d_ctx *ctx, const af3d_particle *pp, const af3d_vec3 *acc,
                                   const af3d_vec3 *anga);
af3d_status af3d_export_particles (af3d_ctx *ctx, af3d_particle *pp, af3d_vec3 *acc,
                                   af3d_vec3 *anga);

/* One step of a caller that keeps the particle array on the host: af3d_import_particles(in,
   acc_in, anga_in), af3d_step(ctx, 1) and af3d_export_particles(out, acc_out, anga_out) in one
   call, with the same results (in and out may be the same arrays; acc_in/anga_in NULL: zero
   accelerations; acc_out/anga_out NULL: not written).  The clumps are imported in input order
   (slot i holds clump i) and the step keeps that order, so each of four parts of the clumps is
   copied in, on a copy stream of its own, while the previous one is converted and predicted,
   and copied out while the force pass of the next one runs (the part nothing overlaps at each
   end holds an eighth of the clumps).  There is no
   counterpart in the reference: it replaces the host-master step of its loop
   (avalanche_hst.cu:668-710 with the particle array on the host) by one call. */
af3d_status af3d_step_host (af3d_ctx *ctx, const af3d_particle *in, const af3d_vec3 *acc_in,
                            const af3d_vec3 *anga_in, af3d_particle *out, af3d_vec3 *acc_out,
                            af3d_vec3 *anga_out);

/* system_par / cell_par passed by value in the reference become context state. */
af3d_status af3d_set_system (af3d_ctx *ctx, const af3d_system_par *sys);
af3d_status af3d_get_system (af3d_ctx *ctx, af3d_system_par *sys);
af3d_status af3d_set_grid (af3d_ctx *ctx, const af3d_cell_par *cell);
af3d_status af3d_get_grid (af3d_ctx *ctx, af3d_cell_par *cell);
af3d_status af3d_set_phase (af3d_ctx *ctx, int phase);

/* ---- batched ensemble: many independent flumes in one context ---------------------------
   The reference runs one flume per process (avalanche_dev.cu:140-158 sizes every array for one
   system).  An ensemble context holds nflumes flumes back to back in clump-id order (flume f
   owns ids [sum npart of flumes < f, + sys[f].npart)), each with its own system_par, Funnel
   and cell grid, stepped together by af3d_step on one stream.  Clumps of different flumes
   never interact.  The flumes share dt and the clock (time); material, geometry and tilt may
   differ.  af3d_create is af3d_create_ensemble with nflumes = 1, and the single-flume calls
   above (set/get_system, set/get_grid) address flume 0. */
af3d_status af3d_create_ensemble (int nflumes, const af3d_system_par *sys, const af3d_funnel *fun,
                                  long ntags, int phase, af3d_ctx **out);
int         af3d_flume_count (af3d_ctx *ctx);
/* fun may be NULL (keep the flume's Funnel).  sys->time sets the shared clock. */
af3d_status af3d_set_flume_system (af3d_ctx *ctx, int flume, const af3d_system_par *sys,
                                   const af3d_funnel *fun);
af3d_status af3d_get_flume_system (af3d_ctx *ctx, int flume, af3d_system_par *sys);
/* Setting the first grid of a context copies it to every flume that has none yet. */
af3d_status af3d_set_flume_grid (af3d_ctx *ctx, int flume, const af3d_cell_par *cell);
af3d_status af3d_get_flume_grid (af3d_ctx *ctx, int flume, af3d_cell_par *cell);

/* cell_dim (cell_dim.cu:7) + grid derivation (avalanche_hst.cu:314-333), on the device, for
   every flume of the context. */
af3d_status af3d_regrid (af3d_ctx *ctx);
/* Door opening: side.x = (LFUNNEL + Lflume) cos(tilt), time = 0, avalanche phase
   (avalanche_hst.cu:607-613). */
af3d_status af3d_open_door (af3d_ctx *ctx);

/* ---- one entry point per reference routine (avalanche_hst.cu:668-710 order) ---------------- */
af3d_status af3d_init_verlet (af3d_ctx *ctx);         /* init_Verlet.cu:11 with a_i, alpha_i     */
af3d_status af3d_advance_time (af3d_ctx *ctx);        /* sys_par.time += dt, avalanche_hst.cu:672*/
af3d_status af3d_rotate_vectors (af3d_ctx *ctx);      /* rotate_vectors.cu:7 (slope frame)       */
af3d_status af3d_clear_forces (af3d_ctx *ctx);        /* clear_forces.cu:8                        */
af3d_status af3d_cell_build (af3d_ctx *ctx);          /* clear_cell + clear_ocup + cell_locate,
                                                         cells.cu:11,26,40                        */
af3d_status af3d_force_hop (af3d_ctx *ctx, int nw);   /* force_hop.cu:9                           */
af3d_status af3d_force_funnel (af3d_ctx *ctx);        /* force_funnel.cu:9                        */
af3d_status af3d_force_fcorners (af3d_ctx *ctx);      /* force_funnel.cu:216                      */
af3d_status af3d_force_walls (af3d_ctx *ctx);         /* force_walls.cu:9                         */
af3d_status af3d_force_part (af3d_ctx *ctx, int sph_id); /* force_part.cu:11; sph_id 1..16, or 0
                                                         for all sixteen in one call              */
af3d_status af3d_force_flume (af3d_ctx *ctx);         /* force_flume.cu:10                        */
af3d_status af3d_get_accel (af3d_ctx *ctx);           /* get_accel.cu:9 -> a_f, alpha_f           */
af3d_status af3d_finish_verlet (af3d_ctx *ctx);       /* finish_Verlet.cu:10 with a_i and a_f     */
af3d_status af3d_swap_accel (af3d_ctx *ctx);          /* avalanche_hst.cu:845-850                 */

/* Fused force pass of the current phase: clear_forces, cell build, every force routine in the
   reference's order, get_accel into a_f (avalanche_hst.cu:678-707; fill :445-464). */
af3d_status af3d_forces (af3d_ctx *ctx);

/* k steps of the current phase, fused and replayed from CUDA graphs, with the reference's
   re-grid every 2000 steps (avalanche_hst.cu:713-748).  Returns the first error status raised
   by the device checks during those steps. */
af3d_status af3d_step (af3d_ctx *ctx, long k);

/* Same steps as af3d_step, enqueued without graphs and with CUDA events between the kernels on
   the context stream; adds the milliseconds of each phase to ms[AF3D_NPROF]:
   0 time advance, 1 init_Verlet + cell keys, 2 cell sort, 3 permutation + neighbour records,
   4 force kernel (contact lists, walls, contacts, bed, get_accel, finish_Verlet), 5 re-grid. */
enum { AF3D_NPROF = 6 };
af3d_status af3d_step_profile (af3d_ctx *ctx, long k, double *ms);
/* Kernels executed on the device by this context so far (graph replays included). */
af3d_status af3d_kernel_launches (af3d_ctx *ctx, long *count);
/* Measured FP64 fused-multiply-add throughput of the current device in TFLOP/s (2 flops per
   DFMA), from a bounded ~0.1 s microbenchmark: the denominator of the FP64 roofline. */
af3d_status af3d_fp64_peak (double *tflops);
/* Self-check of the kernels' integer-pipe FP64 helpers (no counterpart in the reference): the
   conversions to float (to nearest, toward +infinity) and to a 64-bit integer, and the
   finiteness, non-zero and range tests the kernels take from the bit patterns, against the
   hardware instructions, for each x[i]; bad[i] gets one bit per helper that disagreed. */
af3d_status af3d_check_fp64_bits (const double *x, long n, int *bad);

/* ---- adjoint (no counterpart in the reference) --------------------------------------------
   Runs, from the imported state (a_i = alpha_i = 0), the start-up force pass and `steps` exact
   steps (fixed cell grid, no re-grid), and returns per flume f the objective J[f] at the end:
   by default the mass-weighted mean downslope position sum m (x cos(tilt) - z sin(tilt)) / sum m
   of its clumps, or the runout (af3d_set_objective).  With
   any gradient pointer non-NULL it then runs the hand-written adjoint of those steps backwards
   from a tape of C steps (540 B per clump and step: each step's starting state, torque sums,
   clump records and contact item lists), C = min(steps, ckpt_every), halved until the tape and
   the checkpoints fit in the free device memory less 2 GB (the results do not depend on C); the
   last C steps are taped as the forward run goes, each earlier segment of C steps restarts from
   a checkpoint of its starting state (192 B per clump) and is recomputed into the tape.  It
   returns
     param_grad[6 f + k]  dJ[f]/d(kappa_pp, gamma_pp, mu_pp, kappa_pw, gamma_pw, mu_pw)[k] of
                          flume f's system_par
     dr0, dv0, dw0        dJ[f]/d(initial r, v, omega) per clump id, f the clump's flume (the
                          sphere centres follow r and R)
     dR0[9 n]             dJ[f]/d(initial Rmatx, Rmaty, Rmatz) per clump id
   J and param_grad hold af3d_flume_count entries (times 6); an ensemble differentiates all its
   flumes in one backward sweep (they are independent, so the sweep of sum_f J[f] gives each
   flume's own gradients).  Discrete events (cells, contact sets, Coulomb or elastic branch,
   which wall) are held at the forward run's.  Removed clumps carry no gradient.  The context is
   left at the final state of the forward run. */
af3d_status af3d_adjoint (af3d_ctx *ctx, long steps, long ckpt_every, double *J, double *param_grad,
                          af3d_vec3 *dr0, double *dR0, af3d_vec3 *dv0, af3d_vec3 *dw0);
/* No counterpart in the reference.  The objective J[f] af3d_adjoint evaluates and
   differentiates, over flume f's clumps' final downslope positions x = x_rot
   (rotate_vectors.cu:28) with masses m:
     AF3D_OBJ_CENTROID (default)  the deposit centroid, sum m x / sum m (length ignored)
     AF3D_OBJ_RUNOUT              the runout, length * ln(sum m exp(x / length) / sum m): a
                                  mass-weighted soft maximum of x, the front of the deposit as
                                  length -> 0 (a smooth stand-in for the front's position, whose
                                  exact maximum has no useful derivative); length > 0 [cm]. */
af3d_status af3d_set_objective (af3d_ctx *ctx, int objective, double length);

/* No counterpart in the reference.  Captures now, without running anything or changing the
   state, the CUDA graphs the next af3d_step(ctx, k) will replay (up to its first re-grid), so
   that their capture does not fall inside a timed or latency-critical call. */
af3d_status af3d_prepare_steps (af3d_ctx *ctx, long k);
/* No counterpart in the reference.  The fused path keeps the slot order between permutations of
   every plane into (cell, id) order, `steps` apart (even, 2..4096; default 64); one captured
   graph covers one period.  Results do not depend on it (every sum runs in the reference's
   order); it trades the permutation's cost against the drift of the slot order from the
   spatial order. */
af3d_status af3d_set_resort_every (af3d_ctx *ctx, long steps);
/* Autotuner (no counterpart in the reference): times af3d_step with each permutation interval in
   16, 32, 64, 128, 256 (one untimed period, then at least steps_per_trial steps, whole periods)
   and keeps the fastest, returned in *resort_every (may be NULL), with each interval's time per
   step in ms_per_step[5] (may be NULL).  Every step it takes is a
   step of the run -- the trajectory is bit-identical whatever the interval -- so it costs time,
   not accuracy. */
af3d_status af3d_autotune (af3d_ctx *ctx, long steps_per_trial, long *resort_every, double *ms_per_step);
/* The fused force kernel's block (no counterpart in the reference): 64, 96, 128 or 192 threads,
   one clump per thread, the block's clumps pooling their contact items; each runs at the
   resident blocks per SM that measured fastest for it (10, 6, 5 and 3).  Results do not depend
   on it.  A new context starts with the block of 64, 96 and 128 whose last wave is fullest for
   its clump count on the current device; af3d_set_force_block overrides it. */
af3d_status af3d_set_force_block (af3d_ctx *ctx, int block);
af3d_status af3d_get_force_block (af3d_ctx *ctx, int *block);
/* Autotuner over both shape parameters (no counterpart in the reference): af3d_autotune (the
   permutation interval, its times in ms_interval[5]), then each force block (128, 96, 64 and
   192, its times in ms_block[4] in that order) at that interval, one untimed period and whole
   periods timed; keeps the fastest of each.  Every step it takes is a step of the run.  The kernels' remaining shape
   parameters are not tuned: one clump per thread (the block pools its clumps' contact items,
   which replaces a clumps-per-warp choice), and the reference's cell size (a smaller cell
   would miss contacts, a larger one only adds candidates to every walk). */
af3d_status af3d_autotune_shapes (af3d_ctx *ctx, long steps_per_trial, long *resort_every, int *force_block,
                                  double *ms_interval, double *ms_block);

/* Status bits raised on the device since the last call (bitmask of 1 << AF3D_ERR_*); clears. */
af3d_status af3d_get_status (af3d_ctx *ctx, int *flags);

/* ---- diagnostics, indexed by clump id -------------------------------------------------- */
af3d_status af3d_get_forces (af3d_ctx *ctx, af3d_vec3 *force, af3d_vec3 *torque);
af3d_status af3d_get_accels (af3d_ctx *ctx, af3d_vec3 *acc_f, af3d_vec3 *anga_f);
/* Cell of every clump (-1 if not binned) and the (cell, id)-sorted id list of the last build. */
af3d_status af3d_get_cells (af3d_ctx *ctx, long *cell_of_id, long *sorted_ids, long *nbinned);
/* Overlapping sphere pairs (ll, mm, sph_id) of the last cell build, in no particular order;
   active = 1 keeps only pairs with a repulsive normal force.  *count may exceed cap. */
af3d_status af3d_contact_pairs (af3d_ctx *ctx, long *out, long cap, long *count, int active);
/* No counterpart in the reference.  af3d_contact_pairs without any device allocation, for
   callers that must not allocate device memory mid-run (a host whose caching pool already holds
   the GPU's memory; a running simulation that cannot afford the device-wide synchronisation of
   cudaMalloc/cudaFree).  Pairs are staged in a fixed array inside the library's device image:
   cap must lie in [0, 262144] (larger caps are refused with AF3D_ERR_ARG); *count is the total,
   which may exceed cap.  The context's device must be current.  The first call on a device
   looks up the array (set-up): make it before any stream capture.  The staging counter is
   zeroed by each call on the context stream.  All contexts of a device share the array, so
   calls that overlap in time race: serialise them per device. */
af3d_status af3d_contact_pairs_noalloc (af3d_ctx *ctx, long *out, long cap, long *count, int active);
/* Active sphere-sphere contacts summed over the fused force passes (af3d_step, af3d_forces)
   since the previous call; the counter restarts at zero. */
af3d_status af3d_contact_count (af3d_ctx *ctx, long *count);
/* Clumps whose contact item lists overflowed (more than 32 items, 24 partners passing the
   centre test or 48 candidates), summed over the fused force passes since the previous call;
   the counter restarts at zero.  Such a clump's contacts run by the per-clump cell walk, in
   the same summation order (force_part.cu:88-106's walk, one pass per sph_id). */
af3d_status af3d_list_overflows (af3d_ctx *ctx, long *count);

/* Lossless binary checkpoint of a context (no counterpart in the reference, whose
   last_config.dat is %lf text): parameters of every flume, clock, step counter, phase, friction
   variant, FP64 mode, cell grids, the particles and a_i, alpha_i as raw bytes.  Loading it into
   a context of the same shape (clumps, flumes, ntags) continues the run bit for bit as if it
   had not stopped. */
af3d_status af3d_save_checkpoint (af3d_ctx *ctx, const char *path);
af3d_status af3d_load_checkpoint (af3d_ctx *ctx, const char *path);

/* ---- host I/O (no GPU) ----------------------------------------------------------------- */
/* Parse DataInput.dat from an open stream: the first token of each of the next 16 lines, in
   avalanche_hst.cu:34-81's order (the reference reads them from stdin).  The stream is left
   open. */
af3d_status af3d_read_datainput (FILE *fp, af3d_inputs *in);
/* The same from a file path. */
af3d_status af3d_load_datainput (const char *path, af3d_inputs *in);
/* Derived parameters of avalanche_hst.cu:84-102 and :187-195 (time = -1, side.x = HOP_WIDTH). */
af3d_status af3d_derive_system (const af3d_inputs *in, af3d_system_par *sys, af3d_funnel *fun);
/* error_check.cu:3; returns the reference's error number (0 = accepted). */
int         af3d_error_check (const af3d_system_par *sys, char *msg, size_t msglen);
/* last_config.dat writer/reader (avalanche_hst.cu:519-548 / :218-250); %lf text, lossy. */
af3d_status af3d_write_last_config (const char *path, int aval_start, double time, long cc,
                                    long jj, const af3d_particle *pp, long n);
af3d_status af3d_read_last_config (const char *path, int *aval_start, double *time, long *cc,
                                   long *jj, af3d_particle *pp, long n);
/* One output frame of the reference's snapshot files (avalanche_hst.cu:507-586 in the fill
   phase, :750-841 in the avalanche phase), appended to each file whose path is non-NULL:
     xyz_path    the .xyz frame (snapshots_hst.xyz): 4 n + 2 atoms, radius and centre of every
                 sphere, then two ghost atoms that fix the rendered cell
     vel_path    the velocity-field frame (velocities_hst.xyz): r, v.x, w.y per clump + 2 ghosts
     vmean_path  mean_velocity_hst.csv: "time - dt, mean |v|, mean |w|"
     xcm_path    xcm_hst.csv (avalanche phase only): "time - dt, x_cm, z_cm" over sys->tot_mass
   pp in id order (as exported), sys with the current time. */
af3d_status af3d_append_snapshot (const char *xyz_path, const char *vel_path, const char *vmean_path,
                                  const char *xcm_path, const af3d_particle *pp, long n,
                                  const af3d_system_par *sys, int phase);

/* ---- initial-state generators (host; generate_particles.cu, place_particles.cu,
   set_initial_velocity.cu, rannew64.cu, calculate_particle_parameters.cu) ------------------- */
typedef struct { uint64_t seed[250], uy; int np, nq, init; } af3d_rng;
/* rannew64.cu:55-126 with its state in *rng instead of statics: the first draw after seeding
   returns the reference's first draw for that idum. */
void   af3d_rng_seed (af3d_rng *rng, long idum);
double af3d_rng_next (af3d_rng *rng);
/* generate_particles.cu:7-32: density 2.6, every 20th clump rmax, the others rmin. */
void   af3d_generate_particles (af3d_particle *pp, const af3d_system_par *sys);
/* calculate_particle_parameters.cu:10-41 (host version): m = 4 (4/3 pi) rho r^3, I = 112/15 pi rho r^5. */
void   af3d_calculate_particle_parameters (af3d_particle *pp, long n);
/* place_particles.cu:8-90: cubic lattice in the hopper, identity orientation.  Returns
   AF3D_ERR_INPUT when the clumps do not fit (the reference exits). */
af3d_status af3d_place_particles (const af3d_system_par *sys, af3d_particle *pp);
/* set_initial_velocity.cu:7-42 with seed 26752658 on a fresh generator. */
void   af3d_set_initial_velocity (const af3d_system_par *sys, af3d_particle *pp);
/* Sphere centres from rr, R and radius (avalanche_hst.cu:265-293 / init_Verlet.cu:130-142). */
void   af3d_sphere_centres (af3d_particle *pp, long n);
/* Workload generator: clumps on a cubic lattice of the given pitch filling the box
   [lo, hi] (x fastest), each with a uniformly random orientation drawn from rng (Shoemake unit
   quaternion); an orientation whose spheres would overlap an already placed clump or leave the
   box is redrawn (up to max_tries, then the last draw is kept).  Radius, density and mass must
   already be set.  Returns the number of clumps placed (< n when the box is too small). */
long   af3d_lattice_block (af3d_particle *pp, long n, af3d_vec3 lo, af3d_vec3 hi, double pitch,
                           af3d_rng *rng, int max_tries);
/* Workload generator: a pile settled in the box.  Clumps stand in the columns of a square
   lattice of the given pitch (x, y), each with a random orientation from rng (redrawn while a
   sphere would cross a side wall), and are dropped layer by layer: each is lowered until a sphere
   touches the floor z = lo.z or a sphere already placed in its own or a neighbouring column, then
   pressed `overlap` further so its resting contacts carry load.  Radius, density and mass must
   already be set.  Returns the number placed (< n when a clump rises above hi.z). */
long   af3d_lattice_pile (af3d_particle *pp, long n, af3d_vec3 lo, af3d_vec3 hi, double pitch,
                          double overlap, af3d_rng *rng, int max_tries);

#ifdef __cplusplus
}
#endif
#endif
