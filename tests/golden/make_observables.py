"""Generate tests/golden/observables_flume2k.npz: the oracle's long-run observables of the
2,048-clump flume (40 cm x 4 cm, 30 deg, the reference's contact law at dt = 2e-6 s) over
50,000 steps, for 16 seeds of two initial states:
  * "lattice": the release block in the hopper at the moment the door opens (cubic lattice of
    4 mm pitch, random orientations, at rest), which falls freely for the whole 0.1 s;
  * "bed": a dense layer on the flume bed that slides and shears for the whole 0.1 s.
Per seed the runout (95th percentile of the downslope position), the deposit centroid
(mass-weighted mean downslope position) and the mean downslope velocity, at the start and after
the run.  The oracle is the C restatement of the reference's host routines (oracle/), run
single-threaded, one seed per process, with the reference loop's cell_dim re-grid every 2,000
steps.

Run from the repository root after oracle/build.py has built the oracle:
    python tests/golden/make_observables.py [--jobs J]
(about 30 minutes on 8 cores)."""
import argparse
import multiprocessing as mp
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

LAYOUTS = ("lattice", "bed")
SEEDS = tuple(range(1, 17))
STEPS = 50_000
OUT = os.path.join(HERE, "observables_flume2k.npz")


def observables(pp, sys_):
    """(runout, centroid, mean velocity) along the slope: x' = x cos(tilt) - z sin(tilt)."""
    c, s = float(sys_["cost"]), float(sys_["sint"])
    x = pp["rr"][:, 0] * c - pp["rr"][:, 2] * s
    v = pp["vv"][:, 0] * c - pp["vv"][:, 2] * s
    m = pp["mass"]
    return np.array([np.percentile(x, 95), float((m * x).sum() / m.sum()), float(v.mean())])


def _one(job):
    layout, seed = job
    sys.path.insert(0, ROOT)
    from avalancheflume3d_gb300.workloads import flume_2k, flume_state
    from oracle.pyoracle import Oracle, OracleRun
    sys_, fun, pp = flume_state(flume_2k(layout=layout, seed=seed))
    o = Oracle()
    o.set_threads(1)
    run = OracleRun(o, sys_, fun, pp)
    if run.seed_accel() != 0:
        raise RuntimeError("start-up force pass failed: %s seed %d" % (layout, seed))
    before = observables(run.pp, run.sys)
    if run.step(STEPS, cc0=0) != 0:
        raise RuntimeError("oracle run failed: %s seed %d" % (layout, seed))
    return before, observables(run.pp, run.sys)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    jobs = [(layout, seed) for layout in LAYOUTS for seed in SEEDS]
    t0 = time.time()
    with mp.get_context("spawn").Pool(args.jobs) as pool:
        res = pool.map(_one, jobs, chunksize=1)
    before = np.array([b for b, _ in res]).reshape(len(LAYOUTS), len(SEEDS), 3)
    after = np.array([a for _, a in res]).reshape(len(LAYOUTS), len(SEEDS), 3)
    np.savez_compressed(OUT, layouts=np.array(LAYOUTS), seeds=np.array(SEEDS), steps=STEPS,
                        before=before, after=after)
    print("wrote %s in %.0f s" % (OUT, time.time() - t0))
    for i, layout in enumerate(LAYOUTS):
        print(layout, "mean change (runout, centroid, velocity):", (after[i] - before[i]).mean(0))


if __name__ == "__main__":
    main()
