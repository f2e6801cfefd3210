// af3d_avalanche.cpp -- the reference's simulation program (the main of avalanche_hst.cu /
// avalanche_dev.cu) over the engine's C ABI: DataInput.dat in, the reference's output files out.
//
//   1. DataInput.dat (af3d_load_datainput), derived parameters (af3d_derive_system),
//      error_check (af3d_error_check); the reference's initial state: generate_particles,
//      calculate_particle_parameters, place_particles, set_initial_velocity, sphere centres.
//   2. The start-up force pass, then the hopper-filling phase (walls of the hopper closed, time
//      from -1 to 0) until the mean speed falls below v0 / 10 (avalanche_hst.cu:401-601).
//   3. The door opens (side.x = xfinal, time = 0, avalanche_hst.cu:607-613) and the avalanche
//      runs until --t-end, or until the mean speed falls below v0 / 10 after 0.2 s
//      (avalanche_hst.cu:633-857).
//   Every --out-every steps (the reference's 20000) both phases write a frame of
//   snapshots_hst.xyz and velocities_hst.xyz (print flag set), a line of mean_velocity_hst.csv
//   (and of xcm_hst.csv in the avalanche phase) and last_config.dat; the steps in between run
//   through af3d_step (fused, graph-replayed, device re-grid every 2000 steps).
//
// Usage: af3d_avalanche [--input DataInput.dat] [--t-end 2.0] [--out-every 20000]
//   (without --input, or with --input -, the 16 lines of DataInput.dat are read from standard
//   input, as the reference reads them: af3d_avalanche < DataInput.dat)
//                       [--fp exact|fast] [--max-fill-steps N] [--checkpoint PATH]
//                       [--resume PATH]   (a checkpoint written by --checkpoint: the run continues)
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/af3d.h"

namespace {

struct Options {
  std::string input = "-";   // standard input, as avalanche_hst.cu:34-81 reads it
  double t_end = 2.0;   // avalanche_hst.cu:633
  long out_every = 20000;
  bool fast = false;
  long max_fill_steps = -1;   // < 0: no limit
  std::string checkpoint;
  std::string resume;
};

bool parse(int argc, char **argv, Options &o) {
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    auto value = [&](const char *name) -> const char * {
      if (i + 1 >= argc) {
        std::fprintf(stderr, "%s needs a value\n", name);
        return nullptr;
      }
      return argv[++i];
    };
    const char *v = nullptr;
    if (a == "--input" && (v = value("--input"))) o.input = v;
    else if (a == "--t-end" && (v = value("--t-end"))) o.t_end = std::atof(v);
    else if (a == "--out-every" && (v = value("--out-every"))) o.out_every = std::atol(v);
    else if (a == "--fp" && (v = value("--fp"))) o.fast = std::string(v) == "fast";
    else if (a == "--max-fill-steps" && (v = value("--max-fill-steps"))) o.max_fill_steps = std::atol(v);
    else if (a == "--checkpoint" && (v = value("--checkpoint"))) o.checkpoint = v;
    else if (a == "--resume" && (v = value("--resume"))) o.resume = v;
    else {
      std::fprintf(stderr,
                   "usage: af3d_avalanche [--input DataInput.dat] [--t-end S] [--out-every N] "
                   "[--fp exact|fast] [--max-fill-steps N] [--checkpoint PATH] [--resume PATH]\n");
      return false;
    }
    if (!v) return false;
  }
  return o.out_every > 0;
}

bool ok(af3d_status s, const char *what) {
  if (s == AF3D_OK) return true;
  std::fprintf(stderr, "%s: %s\n", what, af3d_last_error());
  return false;
}

// Mean |v| over the clumps, summed in id order (avalanche_hst.cu:563-572).
double mean_speed(const std::vector<af3d_particle> &pp) {
  double vmean = 0.0;
  for (const af3d_particle &p : pp) {
    double vm2 = p.vv.x * p.vv.x;
    vm2 += p.vv.y * p.vv.y;
    vm2 += p.vv.z * p.vv.z;
    vmean += std::sqrt(vm2);
  }
  return pp.empty() ? 0.0 : vmean / (double)pp.size();
}

// Steps from `time` until it reaches `until` (time advances by dt per step), at most `cap`.
long steps_until(double time, double until, double dt, long cap) {
  long k = 0;
  for (double t = time; t < until && k < cap; t += dt) k++;
  return k;
}

}  // namespace

int main(int argc, char **argv) {
  Options o;
  if (!parse(argc, argv, o)) return 2;
  af3d_inputs in;
  const bool from_stdin = o.input == "-";
  if ((from_stdin ? af3d_read_datainput(stdin, &in) : af3d_load_datainput(o.input.c_str(), &in)) != AF3D_OK) {
    std::fprintf(stderr, "cannot read the 16 lines of %s\n", from_stdin ? "DataInput.dat on standard input"
                                                                         : o.input.c_str());
    return 1;
  }
  af3d_system_par sys;
  af3d_funnel fun;
  if (!ok(af3d_derive_system(&in, &sys, &fun), "derived parameters")) return 1;
  char msg[512];
  if (af3d_error_check(&sys, msg, sizeof msg) != 0) {
    std::fprintf(stderr, "%s\n", msg);
    return 1;
  }
  const long n = sys.npart;
  std::vector<af3d_particle> pp((size_t)n);
  af3d_generate_particles(pp.data(), &sys);
  af3d_calculate_particle_parameters(pp.data(), n);
  if (!ok(af3d_place_particles(&sys, pp.data()), "place_particles")) return 1;
  af3d_set_initial_velocity(&sys, pp.data());
  af3d_sphere_centres(pp.data(), n);
  sys.tot_mass = 0.0;
  for (const af3d_particle &p : pp) sys.tot_mass += p.mass;
  std::printf("Total mass: %lf\n", sys.tot_mass);

  af3d_ctx *ctx = nullptr;
  if (!ok(af3d_create(&sys, &fun, in.ntags, AF3D_PHASE_FILL, &ctx), "af3d_create")) return 1;
  struct Destroy {
    af3d_ctx *c;
    ~Destroy() { af3d_destroy(c); }
  } destroy{ctx};
  if (o.fast && !ok(af3d_set_fp_mode(ctx, AF3D_FP_FAST), "af3d_set_fp_mode")) return 1;
  if (o.resume.empty()) {
    if (!ok(af3d_import_particles(ctx, pp.data(), nullptr, nullptr), "import")) return 1;
    if (!ok(af3d_forces(ctx), "start-up force pass") || !ok(af3d_swap_accel(ctx), "swap")) return 1;
  } else {
    // a run saved by --checkpoint continues where it stopped (phase, clock, state, grid)
    if (!ok(af3d_load_checkpoint(ctx, o.resume.c_str()), "resume")) return 1;
    if (o.fast && !ok(af3d_set_fp_mode(ctx, AF3D_FP_FAST), "af3d_set_fp_mode")) return 1;
  }

  long jj = 0;
  // One output frame: the particles back on the host, the snapshot files and last_config.dat.
  auto output = [&](int phase, int aval_start, long cc) -> bool {
    if (!ok(af3d_export_particles(ctx, pp.data(), nullptr, nullptr), "export")) return false;
    if (!ok(af3d_get_system(ctx, &sys), "get_system")) return false;
    const bool print = in.print_flag != 0;
    if (!ok(af3d_append_snapshot(print ? "snapshots_hst.xyz" : nullptr, print ? "velocities_hst.xyz" : nullptr,
                                 "mean_velocity_hst.csv", "xcm_hst.csv", pp.data(), n, &sys, phase),
            "snapshot"))
      return false;
    if (!ok(af3d_write_last_config("last_config.dat", aval_start, sys.time, cc + 1, jj + 1, pp.data(), n),
            "last_config"))
      return false;
    jj++;
    return true;
  };

  // Hopper filling (a resumed run whose door was open -- side.x past the hopper's wall at
  // x = 15, avalanche_hst.cu:607 -- goes straight on with the avalanche)
  if (!ok(af3d_get_system(ctx, &sys), "get_system")) return 1;
  const bool resumed_open = !o.resume.empty() && sys.side.x > 15.0;
  if (!resumed_open) std::printf("Filling hopper...\n");
  long cc = 0;
  while (!resumed_open && sys.time < 0.0 && (o.max_fill_steps < 0 || cc < o.max_fill_steps)) {
    long k = steps_until(sys.time, 0.0, sys.dt, o.out_every);
    if (o.max_fill_steps >= 0) k = std::min(k, o.max_fill_steps - cc);
    if (k <= 0) break;
    if (!ok(af3d_step(ctx, k), "af3d_step")) return 1;
    cc += k;
    if (!output(AF3D_PHASE_FILL, 0, cc)) return 1;
    const double vmean = mean_speed(pp);
    std::printf("Time = %lf s, %ld dt, mean speed %lf\n", sys.time - sys.dt, jj, vmean);
    if (vmean < 0.1 * sys.v0) break;
  }

  // The door opens (unless it was open already); the avalanche runs
  if (!resumed_open) {
    if (!ok(af3d_open_door(ctx), "af3d_open_door")) return 1;
    std::printf("Opening hopper... Avalanche starts!\n");
  }
  if (!ok(af3d_get_system(ctx, &sys), "get_system")) return 1;
  cc = 0;
  while (sys.time < o.t_end) {
    const long k = steps_until(sys.time, o.t_end, sys.dt, o.out_every);
    if (k <= 0) break;
    if (!ok(af3d_step(ctx, k), "af3d_step")) return 1;
    cc += k;
    if (!output(AF3D_PHASE_AVALANCHE, 1, cc)) return 1;
    const double vmean = mean_speed(pp);
    std::printf("Avalanche time = %lf s, %ld dt, mean speed %lf\n", sys.time - sys.dt, jj, vmean);
    if (vmean < 0.1 * sys.v0 && sys.time > 0.2) break;
  }
  if (!o.checkpoint.empty() && !ok(af3d_save_checkpoint(ctx, o.checkpoint.c_str()), "checkpoint")) return 1;
  return 0;
}
