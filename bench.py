#!/usr/bin/env python3
"""Benchmark: clump-steps/s of the fused clump-DEM step on one GB300 (or N replicas).

Workload ``flume262k`` (the 262,144-clump configuration): tetrahedral 4-sphere clumps, sphere
radius 1 mm, density 2.5 g/cm^3, kn = 1e4 N/m (t_coll from the reference's law), restitution 0.5,
mu_pp = 0.5, mu_wall = 0.4, flume 2.0 m x 0.2 m at 35 deg, dt = 2e-6 s, FP64.  Default input
(``--layout bed``): the clumps, each with a uniformly random orientation and zero velocity, are
dropped column by column on a 4 mm lattice onto the flume bed (in the slope frame, between the
side walls, from 1 cm past the funnel exit to 1 cm before the flume end) and onto each other,
then the layer is turned rigidly into the lab frame: a dense avalanche in full flow (~11 clump
layers deep), which gravity keeps loaded on the bed, so the contact density holds over any
timed window.  ``--layout pile`` builds the same packing in the hopper (it falls freely once the
door opens, and its contacts relax within a few tens of steps); ``--layout lattice`` is the
bare release block of the configuration (optionally with the reference's random initial
velocities ``--v0`` and a release ``--preroll``), which has almost no contacts.  Synthetic data;
the state (~350 MB) is larger than L2.

Before timing, the project's autotuner (af3d_autotune_shapes) picks the permutation interval and
the force kernel's block on a context of its own (untimed; ``--no-autotune`` keeps the
defaults), once for the timed FP64 mode and once for the other one.  Timed: exactly K fused steps (graph replays, af3d_step) after W warm-up steps, CUDA
events on the engine's stream, barrier + synchronize on both sides, max over ranks.  Then,
outside the timed region: the other FP64 mode, a profiled pass (CUDA events between the kernels)
for the roofline of the dominant kernel, the end-to-end figures through the C ABI with host
buffers (every step, and once per 2000 steps as the reference's device driver copies), the
2,048- and 524,288-clump configurations, the batched ensemble, the adjoint and the CPU baseline.

``--impl reference`` times the reference's CPU implementation of the step (the oracle port of
the reference's host routines, all host threads) on the same workload (``--cpu-sample M``
takes a section of M clumps instead).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "clump-steps/s"
# Algorithmic HBM bytes of one step: 448 B per clump (state read 192 + constants 32 + state
# write 192 + cell-list traffic 32) plus 8 B per cell.
BYTES_PER_CLUMP = 448
BYTES_PER_CELL = 8


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["engine", "reference"], default="engine")
    p.add_argument("--n", type=int, default=262144, help="clumps (262144 = the benchmark config)")
    p.add_argument("--layout", choices=["bed", "pile", "lattice"], default="bed")
    p.add_argument("--preroll", type=int, default=0, help="untimed release steps of the input")
    p.add_argument("--v0", type=float, default=0.0)
    p.add_argument("--clock-window", type=float, default=1.0,
                   help="seconds of untimed steps before the warm-up, so that the clock samples "
                        "cover the GPU under sustained load (0: none)")
    p.add_argument("--profile-steps", type=int, default=10)
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--e2e-round-trip", type=int, default=2000,
                   help="steps per host round trip of the second end-to-end figure (0: skip)")
    p.add_argument("--cpu-sample", type=int, default=0,
                   help="clumps of the CPU legs: 0 for the whole workload, else the clumps furthest upslope")
    p.add_argument("--cpu-seconds", type=float, default=10.0)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-autotune", dest="autotune", action="store_false",
                   help="skip the autotuner (the timed context keeps the default shapes)")
    p.add_argument("--force-block", type=int, default=0,
                   help="force kernel block of the timed context (64, 96, 128; 0: the default or the "
                        "autotuner's choice)")
    p.add_argument("--no-configs", action="store_true",
                   help="skip the extra configurations (2,048-clump flume, 524,288-clump funnel and hopper)")
    p.add_argument("--fp-mode", choices=["exact", "fast"], default="fast",
                   help="FP64 mode of the timed steps (the other mode is timed beside it)")
    p.add_argument("--no-other-mode", action="store_true", help="do not time the other FP64 mode")
    p.add_argument("--ensemble-flumes", type=int, default=256,
                   help="flumes of the batched-ensemble measurement (0 skips it)")
    p.add_argument("--ensemble-steps", type=int, default=64)
    p.add_argument("--ensemble-seq-flumes", type=int, default=64,
                   help="flumes timed one after another as plain runs (every k-th of the ensemble)")
    p.add_argument("--adjoint-steps", type=int, default=1000,
                   help="steps of the adjoint measurement (0 skips it)")
    p.add_argument("--adjoint-ckpt", type=int, default=1000,
                   help="checkpoint interval of the adjoint (its tape, 540 B per clump and step, holds "
                        "this many steps; at the default the whole run fits and nothing is recomputed)")
    p.add_argument("--adjoint-batch", type=int, default=64,
                   help="parameter samples of the batched (calibration) adjoint (0 skips it)")
    p.add_argument("--adjoint-batch-steps", type=int, default=200)
    p.add_argument("--adjoint-batch-ckpt", type=int, default=200,
                   help="checkpoint interval of the batched adjoint (its tape holds this many steps "
                        "of all samples, 226 GB at the defaults; the library halves it until it fits)")
    p.add_argument("--trace-contacts", type=int, default=0,
                   help="print active contacts every this many pre-roll steps (diagnostic)")
    return p.parse_args()


def workload(args):
    from avalancheflume3d_gb300.workloads import flume_262k, flume_state
    cfg = flume_262k(n=args.n, v0=args.v0, layout=args.layout)
    return cfg, flume_state(cfg)


def config_dict(args, cfg, extra=None):
    d = {"workload": "flume262k" if args.n == 262144 else "flume%d" % args.n,
         "clumps": args.n, "spheres": 4 * args.n, "tilt_deg": cfg.tilt_deg, "flume_m": cfg.Lflume / 100,
         "width_m": cfg.width / 100, "dt_s": cfg.dt, "lattice_mm": cfg.pitch * 10, "v0_cm_s": args.v0,
         "layout": args.layout, "preroll_steps": args.preroll, "load_window_s": args.clock_window,
         "friction": "host (force_part.cu:224)",
         "l2": "state larger than L2 (no flush needed)"}
    if extra:
        d.update(extra)
    return d


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, index: int):
        self.fn = tempfile.NamedTemporaryFile(prefix="af3d_clocks_", suffix=".csv", delete=False).name
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=open(self.fn, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        rows = []
        for line in open(self.fn):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9 and f[1].replace(".", "").isdigit():
                rows.append(f)
        os.unlink(self.fn)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(float(r[1]) for r in rows),
                "sm_max_mhz": max(float(r[2]) for r in rows), "reasons": reasons,
                "samples": len(rows), "window": "untimed load window, warm-up and timed steps"}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def from_profile(key):
    """A per-launch figure of the force kernel (``traffic_bytes_per_launch``,
    ``fp64_flops_per_launch``) from the committed ncu summary, if any."""
    fn = os.path.join(ROOT, "profiles", "lists_forces_flume262k.txt")
    try:
        for line in open(fn):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def traffic_from_profile():
    return from_profile("traffic_bytes_per_launch")


def fp64_line(peak, t_forces, mode):
    """The force kernel's FP64 roofline: its flops per launch (2 DFMA + DADD + DMUL, counted by
    ncu on the fast-mode kernel of this workload) over the event-timed kernel time, against the
    DFMA microbenchmark peak."""
    d = {"peak_tflops": peak, "peak_source": "measured DFMA microbenchmark", "unit": "TFLOP/s"}
    flops = from_profile("fp64_flops_per_launch")
    if flops and t_forces > 0 and mode == "fast":
        d.update({"flops_per_launch": flops, "achieved_tflops": flops / t_forces / 1e12,
                  "frac": flops / t_forces / 1e12 / peak if peak > 0 else None,
                  "flops_source": "profiles/lists_forces_flume262k.txt"})
        # the FP64 pipe also issues compares, conversions and lanes a warp leaves idle: its busy
        # fraction (ncu sm__pipe_fp64_cycles_active) is the bound flops alone understate
        busy = from_profile("fp64_pipe_busy_frac")
        if busy is not None:
            d["pipe_busy_frac"] = busy
    return d


def cpu_sample_state(cfg, sys_, fun, pp, m, acc=None, anga=None):
    """The m clumps furthest upslope (smallest slope-frame x), a full-depth section of the layer,
    as their own system (with their accelerations, when given)."""
    from oracle.pyoracle import SYSTEM_PAR
    s = np.array(sys_, dtype=SYSTEM_PAR).copy()
    s["npart"] = m
    c, si = float(s["cost"]), float(s["sint"])
    xrot = pp["rr"][:, 0] * c - pp["rr"][:, 2] * si
    idx = np.sort(np.argsort(xrot, kind="stable")[:m])
    out = [s, fun, np.ascontiguousarray(pp[idx]).copy()]
    if acc is not None:
        out += [np.ascontiguousarray(acc[idx]), np.ascontiguousarray(anga[idx])]
    return out


def time_cpu(sys_, fun, pp, threads, seconds, acc=None, anga=None, min_steps=2, max_steps=10 ** 6):
    """Steps of the oracle port (the reference's host routines restated in C) timed on the host."""
    from oracle.pyoracle import Oracle, OracleRun
    o = Oracle()
    o.set_threads(threads)
    run = OracleRun(o, sys_, fun, pp, acc=acc, anga=anga)
    if acc is None:
        run.seed_accel()
    t0 = time.perf_counter()
    k = 0
    while k < max_steps and (k < min_steps or time.perf_counter() - t0 < seconds):
        st = run.step(1, cc0=k)
        if st:
            raise RuntimeError("oracle step failed with status %d" % st)
        k += 1
    dt = time.perf_counter() - t0
    return len(pp) * k / dt, k, dt


def _replica_worker(seconds):
    """One single-thread replica of the reference's host routines (the restated port) on the
    2,048-clump flume (dense bed layer), timed for `seconds`."""
    from avalancheflume3d_gb300.workloads import flume_2k, flume_state
    s, f, p = flume_state(flume_2k(layout="bed"))
    return time_cpu(s, f, p, 1, seconds)


def measure_cpu_replicas(procs, seconds):
    """Independent single-thread runs, one per host core, of the 2,048-clump flume: the host's
    throughput ceiling for many small flumes (the ensemble's CPU counterpart).  A spawned pool,
    started before any GPU use of this process."""
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(procs) as pool:
        res = pool.map(_replica_worker, [seconds] * procs)
    return {"value": sum(r[0] for r in res), "unit": "clump-steps/s", "processes": procs,
            "steps_per_process": [r[1] for r in res],
            "sample": "%d independent single-thread runs of the 2,048-clump flume (dense bed layer), "
                      "%.0f s each, all at once" % (procs, seconds)}


def run_reference(args):
    from avalancheflume3d_gb300 import replicas
    if replicas.from_env().rank != 0:
        return
    threads = os.cpu_count() or 1
    cfg, (sys_, fun, pp) = workload(args)
    m = min(args.n, args.cpu_sample) if args.cpu_sample > 0 else args.n
    s, f, q = cpu_sample_state(cfg, sys_, fun, pp, m)[:3] if m < args.n else (sys_, fun, pp)
    from oracle.pyoracle import Oracle, OracleRun
    o = Oracle()
    o.set_threads(threads)
    run = OracleRun(o, s, f, q)
    run.seed_accel()
    pre = min(args.preroll, 200)
    run.step(pre, cc0=0)
    run.step(args.warmup, cc0=pre)
    t0 = time.perf_counter()
    run.step(args.steps, cc0=pre + args.warmup)
    dt = time.perf_counter() - t0
    value = m * args.steps / dt
    if m < args.n:
        sample = ("the %d clumps furthest upslope (a full-depth section of the input) as their own system, "
                  "%d release steps, then %d timed steps" % (m, pre, args.steps))
    else:
        sample = ("the whole workload (%d clumps): start-up force pass, %d warm-up steps, then %d timed steps"
                  % (m, args.warmup, args.steps))
    line = {"metric": METRIC, "value": value, "unit": "clump-steps/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * dt / args.steps * (args.n / m), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(args, cfg, {"cpu_threads": threads}),
            "cpu_baseline": {"value": value, "unit": "clump-steps/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "clump-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "cpu_replicas": measure_cpu_replicas(threads, args.cpu_seconds),
            "reference_gpu": measure_reference_gpu(args, sys_, fun, pp)}
    print(json.dumps(line), flush=True)


def measure_reference_gpu(args, sys_, fun, pp):
    """The reference's OWN device kernels (its *_dev twins, compiled from its sources into
    oracle/_ref/dev) in avalanche_dev.cu:636-693's sequence on cuda:0, on the full workload:
    the start-up pass of avalanche_dev.cu:335-360, W + K steps each checked before launch (the
    reference's cell binning checks no bounds), then the same W + K steps again from a snapshot,
    the last K timed with CUDA events.  31 launches per step, 256 threads per block; the grid
    as cell_dim derives it, with 16 slots per cell."""
    try:
        import torch
        if not torch.cuda.is_available():
            return {"unavailable": "no CUDA device"}
        from oracle import ref_dev
        if not ref_dev.available():
            return {"unavailable": "reference device kernels not built (the reference tree was absent at build time)"}
        from oracle.pyoracle import Oracle, grid_for
        cp = grid_for(pp, sys_, 16, Oracle())
        stream = torch.cuda.current_stream()
        run = ref_dev.RefDeviceRun(sys_, fun, cp, pp, stream=stream.cuda_stream)
        try:
            run.seed_accel()
            snap = run.snapshot()
            run.step_checked(args.warmup + args.steps)
            run.restore(snap)
            run.step(args.warmup)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            l0 = run.launches
            e0.record(stream)
            run.step(args.steps)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            launches = run.launches - l0
        finally:
            run.close()
        return {"value": args.n * args.steps / (ms / 1e3), "unit": "clump-steps/s", "ms_per_step": ms / args.steps,
                "steps": args.steps, "warmup": args.warmup, "launches_per_step": launches / args.steps,
                "kernels": "the reference's *_dev kernels, nvcc -O2 for sm_103a, driven in "
                           "avalanche_dev.cu:636-693's order (friction: the device variant, force_part.cu:487)"}
    except Exception as e:   # the CPU reference line stands on its own
        return {"unavailable": "%s: %s" % (type(e).__name__, e)}


def measure_ensemble(args, stream):
    """Batched ensemble against sequential plain runs, both through af3d_step on this stream.

    Ensemble: ``--ensemble-flumes`` independent flumes of the 2,048-clump geometry with clump
    counts ~ U{1024..16384} and per-flume mu_pp, mu_wall, restitution and slope from a seeded
    rannew64, in one context with a segmented cell list; after a warm-up (which includes the
    device re-grid after the first step and the capture of a 64-step graph) K steps are timed.
    Sequential: every k-th flume of the same ensemble alone in a plain context, the same warm-up
    and K timed steps each, one after another; throughput = their clump-steps / their summed
    times.  Each flume evolves bit-identically in both (the ensemble tests check this)."""
    import torch
    from avalancheflume3d_gb300 import Engine
    from avalancheflume3d_gb300.workloads import ensemble_configs, ensemble_flagged, ensemble_state
    cfgs = ensemble_configs(args.ensemble_flumes, layout=args.layout)
    sys_, fun, pp = ensemble_state(cfgs)
    K = args.ensemble_steps
    warm = K + 1

    def timed(eng):
        eng.prepare_steps(K)   # the graphs are captured before the timed region
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.step(K)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    from avalancheflume3d_gb300 import FP_EXACT, FP_FAST
    mode = FP_FAST if args.fp_mode == "fast" else FP_EXACT
    eng = Engine(sys_, fun, stream=stream.cuda_stream, fp_mode=mode)
    eng.import_particles(pp)
    eng.forces()
    eng.swap_accel()
    tuned = None
    if args.autotune:
        timings = {}
        every, block = eng.autotune_shapes(64, timings)
        tuned = {"resort_every": every, "force_block": block, "ms_per_step": timings}
    eng.step(warm)
    eng.contact_count()
    t_ens = timed(eng)
    contacts = eng.contact_count()
    n_total = len(pp)
    first = eng.first_id.copy()
    # The kernels' own time per step (CUDA events around each kernel group of profiled steps):
    # what a single persistent launch could at best bring the graph-replayed step down to.
    import ctypes as C
    from avalancheflume3d_gb300 import lib
    prof = np.zeros(6)
    lib().af3d_step_profile(eng._h, 16, prof.ctypes.data_as(C.c_void_p))
    prof /= 16
    eng.close()
    del eng
    value = n_total * K / t_ens

    stride = max(1, len(cfgs) // max(1, args.ensemble_seq_flumes))
    seq_units, seq_t = 0, 0.0
    for f in range(0, len(cfgs), stride):
        pp_f = pp[first[f]:first[f + 1]]
        with Engine(sys_[f], fun[f], stream=stream.cuda_stream, fp_mode=mode) as one:
            one.import_particles(pp_f)
            one.forces()
            one.swap_accel()
            one.step(warm)
            seq_t += timed(one)
        seq_units += len(pp_f) * K
    seq = seq_units / seq_t
    return {"flumes": len(cfgs), "clumps": n_total, "steps": K, "warmup": warm,
            "value": value, "unit": "clump-steps/s", "ms_per_step": 1e3 * t_ens / K,
            "contacts_per_step": contacts / K,
            "sequential_plain": {"value": seq, "unit": "clump-steps/s",
                                 "flumes_timed": len(range(0, len(cfgs), stride)),
                                 "what": "every %d-th flume alone in a plain context, one after another"
                                         % stride},
            "speedup_vs_sequential": value / seq,
            "tuned": tuned,
            "kernel_ms_per_step": float(prof.sum()),
            "launch_overhead_ms_per_step": 1e3 * t_ens / K - float(prof.sum()),
            "launch_note": "graph-replayed step time minus the summed kernel-group times of profiled steps: "
                           "the most a single persistent launch could save",
            "flagged_by_error_check": len(ensemble_flagged(cfgs)),
            "graph_steps": 64, "layout": args.layout + " in each hopper, door open at t = 0",
            "geometry": "40 cm x 4 cm flume, reference hopper and funnel; per-flume slope 25-40 deg"}


def _adjoint_cost(sys_, fun, pp, K, ckpt, stream, friction):
    """(forward seconds for K graph-replayed exact steps, adjoint seconds for af3d_adjoint over
    the same K steps from the same state, the adjoint's output)."""
    import torch
    from avalancheflume3d_gb300 import Engine, FP_EXACT

    with Engine(sys_, fun, stream=stream.cuda_stream, fp_mode=FP_EXACT, friction=friction) as eng:
        eng.import_particles(pp)
        eng.forces()
        eng.swap_accel()
        eng.step(K)                      # warm-up
        eng.prepare_steps(K)             # the timed steps' graphs, captured before they are timed
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.step(K)
        e1.record(stream)
        torch.cuda.synchronize()
        t_fwd = e0.elapsed_time(e1) / 1e3
    with Engine(sys_, fun, stream=stream.cuda_stream, friction=friction) as eng:
        eng.import_particles(pp)
        eng.adjoint(min(K, 2 * ckpt), ckpt)   # warm-up
    with Engine(sys_, fun, stream=stream.cuda_stream, friction=friction) as eng:
        eng.import_particles(pp)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = eng.adjoint(K, ckpt)
        torch.cuda.synchronize()
        t_adj = time.perf_counter() - t0
    return t_fwd, t_adj, out


def measure_adjoint(args, stream):
    """Adjoint/forward cost on the adjoint configuration: 32,768 clumps, 80 cm x 4 cm flume at 35
    deg, dense bed layer, exact FP64 (the mode the adjoint differentiates).  Forward: K fused steps
    (graph replay).  Adjoint: af3d_adjoint over the same K steps from the same state (start-up
    pass, forward with checkpoints every C steps, segment recompute, reverse), timed end to end.
    Then the same as a calibration batch: the flume in S copies with sampled (mu_pp, mu_pw,
    restitution) in one ensemble context, every copy's gradients from one backward sweep.

    Both run the device friction variant (force_part.cu:487), whose particle-particle contacts
    take the Coulomb branch when sliding: in the host variant (force_part.cu:224) that branch
    cannot fire for these sphere masses at dt = 2e-6 s, so dJ/dmu_pp is identically zero there.
    The single run also reports the gradients of the runout objective (a soft maximum of the
    downslope positions, length scale 1 cm) from a second adjoint call."""
    from avalancheflume3d_gb300 import Engine, FRICTION_DEV
    from avalancheflume3d_gb300.adjoint import config_gradients
    from avalancheflume3d_gb300.workloads import adjoint_batch, flume_2k, flume_state
    cfg = flume_2k(n=32768, tilt_deg=35.0, Lflume=80.0, layout="bed")
    sys_, fun, pp = flume_state(cfg)
    K = args.adjoint_steps
    t_fwd, t_adj, out = _adjoint_cost(sys_, fun, pp, K, args.adjoint_ckpt, stream, FRICTION_DEV)
    with Engine(sys_, fun, stream=stream.cuda_stream, friction=FRICTION_DEV) as eng:
        eng.import_particles(pp)
        run_out = eng.adjoint(K, args.adjoint_ckpt, runout=1.0)
    res = {"workload": "flume 32,768 clumps, 80 cm x 4 cm at 35 deg, dense bed layer, exact FP64",
           "friction": "device variant (force_part.cu:487); dJ/dmu_pp is identically 0 in the host variant",
           "steps": K, "ckpt_every": args.adjoint_ckpt, "ms_per_step_forward": 1e3 * t_fwd / K,
           "ms_per_step_adjoint": 1e3 * t_adj / K, "adjoint_over_forward": t_adj / t_fwd,
           "what": "adjoint = the whole af3d_adjoint call (forward with checkpoints, segment recompute, "
                   "reverse, gradient gather) per step, over a graph-replayed exact forward step",
           "J": out["J"], "dJ_dparams": out["params"],
           "dJ_dconfig": config_gradients(cfg, out["params"]),
           "runout": {"objective": "1 cm ln(sum m exp(x_rot / 1 cm) / sum m)", "J": run_out["J"],
                      "dJ_dparams": run_out["params"], "dJ_dconfig": config_gradients(cfg, run_out["params"])}}
    S, Kb = args.adjoint_batch, args.adjoint_batch_steps
    if S > 0 and Kb > 0:
        cfgs, bsys, bfun, bpp = adjoint_batch(cfg, S)
        tb_fwd, tb_adj, bout = _adjoint_cost(bsys, bfun, bpp, Kb, args.adjoint_batch_ckpt, stream, FRICTION_DEV)
        g0 = config_gradients(cfgs[0], {k: float(v[0]) for k, v in bout["params"].items()})
        res["batch"] = {
            "samples": S, "clumps": int(len(bpp)), "steps": Kb, "ckpt_every": args.adjoint_batch_ckpt,
            "sampled": "mu_pp ~ U[0.2, 0.8], mu_pw ~ U[0.2, 0.6], restitution ~ U[0.2, 0.8] per copy (rannew64)",
            "ms_per_step_forward": 1e3 * tb_fwd / Kb, "ms_per_step_adjoint": 1e3 * tb_adj / Kb,
            "adjoint_over_forward": tb_adj / tb_fwd,
            "clump_steps_per_s_adjoint": len(bpp) * Kb / tb_adj,
            "clump_steps_per_s_adjoint_single": cfg.n * K / t_adj,
            "J_range": [float(bout["J"].min()), float(bout["J"].max())],
            "dJ_dconfig_sample0": g0}
    return res


def measure_config(name, cfg, steps, warmup, mode, stream, cpu_seconds=0.0):
    """One more configuration, timed like the headline (graph-replayed af3d_step, CUDA events on
    the engine's stream, after `warmup` steps and a start-up force pass): ms per step, clump-
    and contact-throughput, the per-kernel split of a profiled pass and the force kernel's HBM
    roofline (B = 448 N + 8 C per launch).  With cpu_seconds > 0 also the oracle port on one
    host core on the same state (a bounded window of steps)."""
    import ctypes as C
    import torch
    from avalancheflume3d_gb300 import Engine, lib
    from avalancheflume3d_gb300.workloads import flume_state
    sys_, fun, pp = flume_state(cfg)
    with Engine(sys_, fun, ntags=cfg.ntags, stream=stream.cuda_stream, fp_mode=mode) as eng:
        eng.import_particles(pp)
        eng.forces()
        eng.swap_accel()
        eng.step(warmup)
        eng.prepare_steps(steps)
        eng.contact_count()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        eng.step(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        contacts = eng.contact_count()
        ncell3 = int(eng.get_grid()["ncell3"])
        block = eng.force_block()
        names = ["time_advance", "predict_keys", "cell_sort", "permute_records", "fused_forces", "regrid"]
        prof = np.zeros(len(names))
        nprof = max(2, min(10, steps))
        lib().af3d_step_profile(eng._h, nprof, prof.ctypes.data_as(C.c_void_p))
        prof /= nprof
    peaks, peak_kind = measured_peaks()
    t_forces = prof[names.index("fused_forces")] / 1e3
    alg = BYTES_PER_CLUMP * len(pp) + BYTES_PER_CELL * ncell3
    out = {"workload": name, "clumps": len(pp), "cells": ncell3, "steps": steps, "warmup": warmup,
           "value": len(pp) * steps / (ms / 1e3), "unit": "clump-steps/s", "ms_per_step": ms / steps,
           "contacts_per_step": contacts / steps, "contacts_per_s": contacts / (ms / 1e3),
           "force_block": block, "phase_ms": {k: float(v) for k, v in zip(names, prof)},
           "roofline": {"kernel": "k_lists_forces", "algorithmic_bytes_per_launch": alg,
                        "achieved": alg / t_forces / 1e9 if t_forces > 0 else None, "unit": "GB/s",
                        "peak": peaks.get("hbm_gbs"), "peak_source": peak_kind,
                        "frac": alg / t_forces / 1e9 / peaks["hbm_gbs"] if t_forces > 0 else None}}
    if cpu_seconds > 0:
        val, k, dt = time_cpu(sys_, fun, pp, 1, cpu_seconds)
        out["cpu_baseline"] = {"value": val, "unit": "clump-steps/s", "cores": 1, "kind": "port",
                               "sample": "the whole state, %d steps in %.1f s, 1 thread" % (k, dt)}
    return out


def time_other_mode(eng, modes, other, args, stream, R, dev, world, tuned=None):
    """K steps of the other FP64 mode on the same state (after the timed region), with the
    shapes the autotuner picked for that mode (`tuned`) when it ran."""
    import torch
    from avalancheflume3d_gb300 import replicas
    eng.set_fp_mode(modes[other])
    if tuned:
        eng.set_resort_every(tuned["resort_every"])
        eng.set_force_block(tuned["force_block"])
    eng.step(2)
    eng.prepare_steps(args.steps)
    torch.cuda.synchronize()
    o0, o1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    o0.record(stream)
    eng.step(args.steps)
    o1.record(stream)
    torch.cuda.synchronize()
    ms_other = replicas.max_over_ranks(R, o0.elapsed_time(o1), dev)
    line = {"fp_mode": other, "value": world * args.n * args.steps / (ms_other / 1e3),
            "ms_per_step": ms_other / args.steps, "steps": args.steps, "force_block": eng.force_block()}
    if tuned:
        line["tuned"] = tuned
    return line


def run_engine(args):
    import torch
    from avalancheflume3d_gb300 import replicas
    R = replicas.from_env()
    rank, world, local = R.rank, R.world, R.local
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    replicas.init(R, "nccl", dev)
    from avalancheflume3d_gb300 import Engine, PARTICLE, lib
    import ctypes as C

    cfg, (sys_, fun, pp) = workload(args)
    stream = torch.cuda.current_stream()
    from avalancheflume3d_gb300 import FP_EXACT, FP_FAST
    modes = {"exact": FP_EXACT, "fast": FP_FAST}
    def make_engine(trace_preroll=False):
        """A context at the timed run's starting state: the input, the start-up force pass into
        a_i (avalanche_hst.cu:366-384) and the pre-roll."""
        e = Engine(sys_, fun, stream=stream.cuda_stream, fp_mode=modes[args.fp_mode])
        e.import_particles(pp)
        e.forces()
        e.swap_accel()
        if args.preroll:
            if trace_preroll and args.trace_contacts:
                trace = []
                e.contact_count()
                done = 0
                while done < args.preroll:
                    k = min(args.trace_contacts, args.preroll - done)
                    e.step(k)
                    done += k
                    trace.append((done, e.contact_count() / k))
                if rank == 0:
                    print("contacts per step during the pre-roll:", trace, file=sys.stderr, flush=True)
            else:
                e.step(args.preroll)
        return e

    # Clocks are sampled every 200 ms from the start of an untimed load window (--clock-window)
    # to the end of the timed region, all under load: the timed window alone is shorter than one
    # sampling period.  The load window runs on its own context, so the timed steps start from
    # the same state whatever the speed of the code.
    clocks = ClockSampler(local)
    tuned = None
    if args.clock_window > 0 or args.autotune:
        with make_engine() as warm:
            t_end = time.perf_counter() + args.clock_window
            if args.autotune:
                # the project's autotuner on a context of its own (untimed): the permutation
                # interval, then the force kernel's block, each the fastest on real steps
                timings = {}
                every, block = warm.autotune_shapes(64, timings)
                tuned = {"resort_every": every, "force_block": block, "ms_per_step": timings,
                         "what": "af3d_autotune_shapes on the workload's own steps before the timed run"}
            while time.perf_counter() < t_end:
                warm.step(64)
                torch.cuda.synchronize()
    # the other FP64 mode's shapes, tuned the same way on a context of its own (untimed): the
    # exact mode's heavier contact law favours a larger block pool
    other = "exact" if args.fp_mode == "fast" else "fast"
    tuned_other = None
    if args.autotune and not args.no_other_mode:
        with make_engine() as warm:
            warm.set_fp_mode(modes[other])
            timings = {}
            every, block = warm.autotune_shapes(64, timings)
            tuned_other = {"resort_every": every, "force_block": block, "ms_per_step": timings}
    eng = make_engine(trace_preroll=True)
    if tuned:
        eng.set_resort_every(tuned["resort_every"])
        eng.set_force_block(tuned["force_block"])
    if args.force_block:
        eng.set_force_block(args.force_block)
    eng.step(args.warmup)
    eng.prepare_steps(args.steps)   # capture the timed steps' graphs now (nothing runs)
    grid = eng.get_grid()
    ncell3 = int(grid["ncell3"])
    eng.contact_count()   # restart the counter
    launches0 = C.c_long()
    lib().af3d_kernel_launches(eng._h, C.byref(launches0))

    def barrier():
        replicas.barrier(R)

    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    eng.step(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    eng_block = eng.force_block()
    contacts = eng.contact_count()
    launches1 = C.c_long()
    lib().af3d_kernel_launches(eng._h, C.byref(launches1))
    ms = replicas.max_over_ranks(R, ms, dev)
    ms_step = ms / args.steps
    value = world * args.n * args.steps / (ms / 1e3)

    # The other FP64 mode on the same state, same step count (outside the timed region).
    other_line = None
    if not args.no_other_mode:
        other_line = time_other_mode(eng, modes, other, args, stream, R, dev, world, tuned_other)
    eng.set_fp_mode(modes[args.fp_mode])
    eng.set_force_block(eng_block)
    if tuned:
        eng.set_resort_every(tuned["resort_every"])

    # Roofline of the dominant kernel from CUDA events between the kernels (profiled steps after
    # the timed region, same stream).
    names = ["time_advance", "predict_keys", "cell_sort", "permute_records", "fused_forces", "regrid"]
    prof = np.zeros(len(names))
    lib().af3d_step_profile(eng._h, args.profile_steps, prof.ctypes.data_as(C.c_void_p))
    prof /= args.profile_steps
    peaks, peak_kind = measured_peaks()
    t_forces = prof[names.index("fused_forces")] / 1e3
    alg = BYTES_PER_CLUMP * args.n + BYTES_PER_CELL * ncell3
    achieved = alg / t_forces / 1e9 if t_forces > 0 else None
    fp64 = C.c_double()
    lib().af3d_fp64_peak(C.byref(fp64))

    # End to end through the C ABI with pinned host buffers: import (H2D), one step, export (D2H).
    e2e = None
    if args.e2e_steps > 0:
        h_pp = torch.empty(args.n * PARTICLE.itemsize, dtype=torch.uint8, pin_memory=True)
        h_acc = torch.empty(args.n * 3, dtype=torch.float64, pin_memory=True)
        h_anga = torch.empty(args.n * 3, dtype=torch.float64, pin_memory=True)
        npp = h_pp.numpy().view(PARTICLE)
        na, nal = h_acc.numpy().reshape(-1, 3), h_anga.numpy().reshape(-1, 3)
        p_, a_, al_ = eng.export_particles()
        npp[:] = p_
        na[:] = a_
        nal[:] = al_
        ptrs = [a.ctypes.data_as(C.c_void_p) for a in (npp, na, nal)]

        def e2e_step():
            st = lib().af3d_step_host(eng._h, *ptrs, *ptrs)
            if st != 0:
                raise RuntimeError("af3d_step_host failed: %d" % st)

        for _ in range(3):   # untimed warm-up of the same round trip
            e2e_step()
        barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            e2e_step()
        torch.cuda.synchronize()
        barrier()
        dt = replicas.max_over_ranks(R, time.perf_counter() - t0, dev)
        nbytes = args.n * (PARTICLE.itemsize + 48)
        e2e = {"value": world * args.n * args.e2e_steps / dt, "unit": "clump-steps/s",
               "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
               "what": "per step: af3d_step_host on pinned host arrays (import of the AoS + a_i, one "
                       "step, export of the AoS + a_i in place; the copies of each quarter of the "
                       "clumps overlap the work on the others)"}
        # The reference's own device driver copies the particles back every 2000 steps
        # (avalanche_dev.cu:741, for its re-grid and output): the same round trip through the C
        # ABI once per 2000 fused steps, beside the per-step contract above.
        if args.e2e_round_trip > 0:
            K = args.e2e_round_trip
            p_ptr, a_ptr, al_ptr = ptrs

            def trip():
                for fn, argv in (("af3d_import_particles", (eng._h, p_ptr, a_ptr, al_ptr)),
                                 ("af3d_step", (eng._h, K)),
                                 ("af3d_export_particles", (eng._h, p_ptr, a_ptr, al_ptr))):
                    st = getattr(lib(), fn)(*argv)
                    if st != 0:
                        raise RuntimeError("%s failed: %d" % (fn, st))

            trip()   # untimed: its graphs are captured here
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            trip()
            torch.cuda.synchronize()
            dtk = replicas.max_over_ranks(R, time.perf_counter() - t0, dev)
            e2e["round_trip"] = {"value": world * args.n * K / dtk, "unit": "clump-steps/s", "steps_per_trip": K,
                                 "h2d_bytes_per_trip": nbytes, "d2h_bytes_per_trip": nbytes,
                                 "what": "import of the AoS + a_i, %d fused steps (af3d_step), export of the "
                                         "AoS + a_i, as the reference's device driver copies every 2000 steps" % K}

    configs = {}
    if world == 1 and not args.no_configs:
        from avalancheflume3d_gb300.workloads import flume_2k, funnel_524k
        mode = modes[args.fp_mode]
        configs["flume2k"] = measure_config(
            "flume2k: 2,048 clumps, 40 cm x 4 cm flume at 30 deg, dense bed layer", flume_2k(layout="bed"),
            1000, 20, mode, stream, 0.0 if args.no_cpu else min(5.0, args.cpu_seconds))
        configs["funnel524k"] = measure_config(
            "funnel524k: 524,288 polydisperse clumps (size factor U[0.8, 1.2]), reference hopper, funnel and "
            "40 cm x 4 cm flume at 30 deg; half in the hopper, half on the funnel and flume bed", funnel_524k(),
            args.steps, args.warmup, mode, stream)

    ens = None
    if world == 1 and args.ensemble_flumes > 0:
        ens = measure_ensemble(args, stream)
    adj = None
    if world == 1 and args.adjoint_steps > 0:
        adj = measure_adjoint(args, stream)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        p_, a_, al_ = eng.export_particles()
        m = min(args.cpu_sample, args.n) if args.cpu_sample > 0 else args.n
        if m < args.n:
            s, f, q, qa, qal = cpu_sample_state(cfg, eng.get_system(), fun, p_, m, a_, al_)
            what = "the %d clumps furthest upslope in the timed state (a full-depth section) as their own system" % m
        else:
            s, f, q, qa, qal = eng.get_system(), fun, p_, a_, al_
            what = "the whole timed state (%d clumps)" % m
        val, k, dt = time_cpu(s, f, q, 1, args.cpu_seconds, acc=qa, anga=qal)
        cpu = {"value": val, "unit": "clump-steps/s", "cores": 1, "kind": "port",
               "sample": "%s, %d steps in %.1f s, 1 thread" % (what, k, dt)}

    eng.close()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "clump-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": config_dict(args, cfg, {"parallelism": "replicas" if world > 1 else "single",
                                              "cells": ncell3, "fp_mode": args.fp_mode,
                                              "graphs": "captured before the timed steps "
                                                        "(af3d_prepare_steps)"}),
            "other_fp_mode": other_line,
            "contacts_per_s": world * contacts / (ms / 1e3),
            "contacts_per_step": contacts / args.steps,
            "e2e": e2e,
            "gpu_launches": int(launches1.value - launches0.value),
            "roofline": {"bound": "hbm", "kernel": "k_lists_forces", "achieved": achieved,
                         "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                         "frac": (achieved / peaks["hbm_gbs"]) if achieved else None,
                         "peak_source": peak_kind, "traffic": traffic_from_profile(),
                         "algorithmic_bytes_per_launch": alg,
                         "kernel_ms": prof[names.index("fused_forces")], "note": "FP64-issue bound; see fp64"},
            "fp64": fp64_line(fp64.value, t_forces, args.fp_mode),
            "phase_ms": {k: float(v) for k, v in zip(names, prof)},
            "tuned": tuned,
            "force_block": eng_block,
            "configs": configs or None,
            "ensemble": ens,
            "adjoint": adj,
            "cpu_baseline": cpu,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    replicas.finalize(R)


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_engine(args)


if __name__ == "__main__":
    main()
