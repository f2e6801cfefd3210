"""Pin the oracle restatement against the reference's own routines compiled from source.

Every routine of the step, and whole steps of both phases, must give BIT-IDENTICAL results
(same state in, same bytes out).  Skipped where the reference tree is absent; the committed
fixtures of tests/golden/ (checked in test_golden.py) carry the pin to other machines.
"""
import numpy as np
import pytest

from oracle.pyoracle import FRICTION_HST, PHASE_AVALANCHE, PHASE_FILL
from tests.states import Work, flume_system, grid_from_state, run_forces, run_step, sorted_order, wall_state
from oracle.pyoracle import dense_state


def _same(a, b):
    return np.asarray(a).tobytes() == np.asarray(b).tobytes()


def _pair(oracle, reference, n, seed, state="wall", time=0.001, side_x=None):
    sys, fun = flume_system(n, time=time, side_x=side_x)
    if state == "wall":
        pp = wall_state(n, seed, sys)
    else:
        pp = dense_state(n, seed, sys, box=(1.0, 8.0, 26.0))
    cp = grid_from_state(pp, sys, 9, reference)
    return sys, fun, cp, pp


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_routines_bit_identical(oracle, reference, seed):
    n = 600
    sys, fun, cp, pp = _pair(oracle, reference, n, seed)
    rng = np.random.default_rng(seed)
    acc = rng.normal(size=(n, 3)) * 100.0
    anga = rng.normal(size=(n, 3)) * 1000.0
    ai = rng.normal(size=(n, 3))
    results = {}
    for name, lib in (("orc", oracle), ("ref", reference)):
        p = pp.copy()
        w = Work(n, cp)
        lib.init_verlet(acc, anga, sys, p)
        lib.rotate_vectors(p, sys)
        run_forces(lib, sys, fun, cp, p, w, PHASE_AVALANCHE, FRICTION_HST)
        F, T = w.F.copy(), w.T.copy()
        per = {}
        for rname in ("hop0", "hop1", "hop2", "funnel", "fcorners", "walls", "flume"):
            f, t = np.zeros((n, 3)), np.zeros((n, 3))
            if rname.startswith("hop"):
                lib.force_hop(f, t, sys, p, int(rname[3]))
            elif rname == "funnel":
                lib.force_funnel(f, t, sys, p, fun)
            elif rname == "fcorners":
                lib.force_fcorners(f, t, sys, fun, p)
            elif rname == "walls":
                lib.force_walls(f, t, sys, p)
            else:
                lib.force_flume(f, t, sys, p)
            per[rname] = (f, t)
        af, alf = np.zeros((n, 3)), np.zeros((n, 3))
        lib.get_accel(F, T, af, alf, sys, p)
        lib.finish_verlet(ai, ai * 2, af, alf, sys, p)
        results[name] = (p, F, T, per, af, alf, sorted_order(cp, w))
    o, r = results["orc"], results["ref"]
    assert _same(o[0], r[0]), "particle state after init_Verlet/rotate/finish_Verlet"
    assert _same(o[1], r[1]) and _same(o[2], r[2]), "force/torque after the full force pass"
    for k in o[3]:
        assert _same(o[3][k][0], r[3][k][0]) and _same(o[3][k][1], r[3][k][1]), k
        # every boundary routine must be exercised by the wall state
        assert np.count_nonzero(np.abs(o[3][k][0]).sum(1)) > 0 or k in ("hop2",), k
    assert _same(o[4], r[4]) and _same(o[5], r[5]), "get_accel"
    assert np.array_equal(o[6][0], r[6][0]) and np.array_equal(o[6][1], r[6][1]), "cell order"


def test_part_contacts_present(oracle, reference):
    n = 600
    sys, fun, cp, pp = _pair(oracle, reference, n, 7, state="dense")
    w = Work(n, cp)
    run_forces(oracle, sys, fun, cp, pp, w, PHASE_AVALANCHE)
    pairs = oracle.contact_pairs(w.cell_vec, w.nocup, pp, sys, cp)
    assert len(pairs) > n // 2  # a dense state has many sphere contacts


@pytest.mark.parametrize("phase", [PHASE_FILL, PHASE_AVALANCHE])
def test_steps_bit_identical(oracle, reference, phase):
    n = 500
    time = -0.01 if phase == PHASE_FILL else 0.0
    sys, fun, cp, pp = _pair(oracle, reference, n, 11, state="dense" if phase == PHASE_FILL else "wall",
                             time=time)
    states = {}
    for name, lib in (("orc", oracle), ("ref", reference)):
        s = sys.copy()
        p = pp.copy()
        w = Work(n, cp)
        run_forces(lib, s, fun, cp, p, w, phase)   # seed a_i as the reference start-up does
        w.a_i, w.a_f = w.a_f, w.a_i
        w.al_i, w.al_f = w.al_f, w.al_i
        for _ in range(20):
            run_step(lib, s, fun, cp, p, w, phase)
        states[name] = (p, w.a_i, w.al_i, s)
    o, r = states["orc"], states["ref"]
    assert _same(o[0], r[0]) and _same(o[1], r[1]) and _same(o[2], r[2])


def test_removed_clumps(oracle, reference):
    """Clumps past side.x at time > 0 are skipped (radius zeroed, v zeroed, not binned)."""
    n = 400
    sys, fun = flume_system(n, time=0.01)
    pp = wall_state(n, 5, sys)
    sys["side"][0] = float(np.median(pp["rr"][:, 0]))
    cp = grid_from_state(pp, sys, 9, reference)
    out = {}
    for name, lib in (("orc", oracle), ("ref", reference)):
        s, p, w = sys.copy(), pp.copy(), Work(n, cp)
        for _ in range(3):
            run_step(lib, s, fun, cp, p, w, PHASE_AVALANCHE)
        out[name] = (p, w.a_i)
    assert _same(out["orc"][0], out["ref"][0]) and _same(out["orc"][1], out["ref"][1])
    assert (out["orc"][0]["radius"] == 0).sum() > n // 4


def test_cell_dim_and_grid(oracle, reference):
    n = 300
    sys, fun, cp, pp = _pair(oracle, reference, n, 3)
    for lib in (oracle, reference):
        hi, lo = lib.cell_dim(pp, sys)
        ho, loo = reference.cell_dim(pp, sys)
        assert _same(hi, ho) and _same(lo, loo)
    cpo = cp.copy()
    oracle.grid_from_bbox(cpo, sys)
    assert _same(cpo, cp)
