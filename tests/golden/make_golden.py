"""Generate the golden fixtures of tests/golden/ from the reference's OWN host routines.

Run where the reference tree exists (it is compiled from source into oracle/_ref by
oracle/build.py):  python tests/golden/make_golden.py

Each fixture is a seeded clump state (the reference's `particle` layout) with its system_par,
Funnel and cell_par, and what the reference computes from it:
  * one force pass of the phase (clear_forces, cells, every force routine, get_accel):
    force, torque, a_f, alpha_f; the cell slot table as (cell, id)-sorted ids and cells; the
    overlapping sphere pairs (enumerated by the restatement with the staged test of
    force_part.cu:140-157; the reference has no enumeration routine of its own)
  * the state and a_i after 1 and after 100 steps of the reference loop
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.pyoracle import (PHASE_AVALANCHE, PHASE_FILL, Oracle, Reference, dense_state)  # noqa: E402
from tests.states import Work, flume_system, grid_from_state, run_forces, run_step, sorted_order, wall_state  # noqa: E402

CASES = {
    "wall_avalanche": dict(kind="wall", n=180, seed=101, phase=PHASE_AVALANCHE, time=0.0),
    "dense_fill": dict(kind="dense", n=160, seed=202, phase=PHASE_FILL, time=-0.5),
    "dense_avalanche": dict(kind="dense", n=200, seed=303, phase=PHASE_AVALANCHE, time=0.0),
}


def make_case(ref, kind, n, seed, phase, time):
    sys_, fun = flume_system(n, time=time)
    pp = wall_state(n, seed, sys_) if kind == "wall" else dense_state(n, seed, sys_, box=(1.0, 8.0, 26.0))
    cp = grid_from_state(pp, sys_, 9, ref)
    out = {"sys": sys_.copy(), "fun": fun.copy(), "cell": cp.copy(), "pp": pp.copy(), "phase": phase}
    w = Work(n, cp)
    p = pp.copy()
    run_forces(ref, sys_, fun, cp, p, w, phase)
    out["force"], out["torque"] = w.F.copy(), w.T.copy()
    out["acc_f"], out["anga_f"] = w.a_f.copy(), w.al_f.copy()
    ids, cells = sorted_order(cp, w)
    out["sorted_ids"], out["sorted_cells"] = ids, cells
    out["pairs"] = Oracle().contact_pairs(w.cell_vec, w.nocup, p, sys_, cp)
    # the reference loop: seed a_i with the start-up force pass, then steps
    w.a_i, w.a_f = w.a_f, w.a_i
    w.al_i, w.al_f = w.al_f, w.al_i
    out["acc_i0"], out["anga_i0"] = w.a_i.copy(), w.al_i.copy()
    s = sys_.copy()
    for k in range(100):
        run_step(ref, s, fun, cp, p, w, phase)
        if k == 0:
            out["pp_1"], out["acc_1"] = p.copy(), w.a_i.copy()
    out["pp_100"], out["acc_100"], out["time_100"] = p.copy(), w.a_i.copy(), float(s["time"])
    return out


def main():
    ref = Reference()
    for name, kw in CASES.items():
        out = make_case(ref, **kw)
        fn = os.path.join(HERE, name + ".npz")
        np.savez_compressed(fn, **{k: np.asarray(v) for k, v in out.items()})
        print(fn, os.path.getsize(fn), "bytes,", len(out["pairs"]), "overlapping sphere pairs")


if __name__ == "__main__":
    main()
