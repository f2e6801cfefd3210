"""Parity at the benchmarked sizes, on the very states bench.py times, against the pinned CPU
oracle (run with every host thread):

  * flume262k: 262,144 clumps of the 2.0 m x 0.2 m flume at 35 deg, the dense bed layer
    (workloads.flume_262k(layout="bed"), 4.19 M cells), the headline workload;
  * funnel524k: 524,288 polydisperse clumps (size factor U[0.8, 1.2]) in the reference's hopper,
    funnel and 40 cm x 4 cm flume at 30 deg, half in the hopper, half on the funnel and flume bed
    (workloads.funnel_524k), touching every boundary routine.

Two states of each: the input as the generator builds it, and the state the timed steps start
from, 5 steps later (bench.py's warm-up; the oracle's steps from the input).  In the input every
clump rests exactly on its support with zero velocity, so every contact's compression is at the
rounding level of the coordinates (~1e-14 cm) and its force is rounding noise; 5 steps later
gravity has loaded the contacts, and forces are defined to far more than 1e-10.

Bars, as for the small states (force_part.cu:11-266, cells.cu:40-111, avalanche_hst.cu:668-710):
  * exact FP64 mode, both states: one force pass's F, T, a and alpha bit-identical to the oracle
    (both friction variants on the input); the cell of every clump, the (cell, id) order and the
    contact-pair sets (all overlapping sphere pairs, and the active ones) identical;
  * fast FP64 mode, the timed state: F, T, a and alpha within 1e-10 relative per clump (a clump
    whose net force nearly cancels is measured against 1e-6 of the largest norm instead);
    contact-pair sets identical to the exact mode's;
  * 100 fused steps from the timed state (af3d_step, with the device re-grid after the first) in
    either mode: every position, velocity, spin, rotation row and sphere centre within 1e-8
    relative.
"""
import os

import numpy as np
import pytest

from oracle.pyoracle import FRICTION_DEV, FRICTION_HST, OracleRun

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-10
TRAJ_RTOL = 1e-8
STEPS = 100
WARMUP = 5


@pytest.fixture(scope="module")
def af3d():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    af3d.lib()
    return af3d


def _config(name):
    from avalancheflume3d_gb300.workloads import flume_262k, funnel_524k
    return {"flume262k": lambda: flume_262k(layout="bed"), "funnel524k": funnel_524k}[name]()


class Case:
    """One workload: its input state, its state after the warm-up steps (with a_i), the oracle's
    force passes on either and the oracle's trajectory from the warmed state."""

    def __init__(self, name, oracle):
        from avalancheflume3d_gb300.workloads import flume_state
        oracle.set_threads(os.cpu_count() or 1)
        self.o = oracle
        self.cfg = _config(name)
        self.sys, self.fun, self.pp = flume_state(self.cfg)
        self.n = len(self.pp)
        run = OracleRun(oracle, self.sys, self.fun, self.pp, ntags=self.cfg.ntags)
        assert run.seed_accel() == 0
        assert run.step(WARMUP, cc0=0) == 0
        self.warm = (run.sys.copy(), run.pp.copy(), run.acc_i[0].copy(), run.acc_i[1].copy())
        self._forces = {}
        self._traj = None

    def state(self, when):
        """(system_par, particles, a_i, alpha_i) of the input or of the warmed state."""
        if when == "input":
            return self.sys, self.pp, None, None
        return self.warm

    def forces(self, when="warm", friction=FRICTION_HST):
        key = (when, friction)
        if key not in self._forces:
            sys, pp, _, _ = self.state(when)
            run = OracleRun(self.o, sys, self.fun, pp, ntags=self.cfg.ntags)
            assert run.forces(variant=friction) == 0
            a, al = run.acc_f
            self._forces[key] = run, (run.bufs["F"].copy(), run.bufs["T"].copy(), a.copy(), al.copy())
        return self._forces[key]

    def trajectory(self):
        if self._traj is None:
            sys, pp, a, al = self.warm
            run = OracleRun(self.o, sys, self.fun, pp, ntags=self.cfg.ntags, acc=a, anga=al)
            assert run.step(STEPS, cc0=0) == 0
            self._traj = run.pp.copy(), run.acc_i[0].copy()
        return self._traj

    def engine(self, af3d, mode, when="warm", friction=FRICTION_HST, cp=None):
        sys, pp, a, al = self.state(when)
        eng = af3d.Engine(sys, self.fun, ntags=self.cfg.ntags, friction=friction, fp_mode=mode)
        if cp is not None:
            eng.set_grid(cp)
        eng.import_particles(pp, a, al)
        return eng


_CASES = {}


@pytest.fixture(scope="module", params=["flume262k", "funnel524k"])
def case(request, oracle):
    if request.param not in _CASES:
        _CASES.clear()          # one full-size state in host memory at a time
        _CASES[request.param] = Case(request.param, oracle)
    return _CASES[request.param]


def _rel_err(got, want):
    norm = np.linalg.norm(want, axis=1)
    floor = 1e-6 * max(float(norm.max()), 1e-300)
    return float(np.max(np.linalg.norm(got - want, axis=1) / np.maximum(norm, floor)))


def _sorted_slots(run):
    """(cell, id)-sorted ids and their cells from the oracle's slot table (cells.cu:40-111)."""
    ntags = int(run.cp["ntags"])
    nocup = run.nocup[:int(run.cp["ncell3"])]
    table = run.cell_vec[:len(nocup) * ntags].reshape(len(nocup), ntags)
    used = np.arange(ntags)[None, :] < nocup[:, None]
    cells = np.broadcast_to(np.arange(len(nocup))[:, None], used.shape)[used]
    return table[used], cells


def _pair_keys(pairs):
    """Each (clump, partner, sph_id) triple as one sortable integer."""
    p = np.asarray(pairs, dtype=np.int64)
    return np.sort((p[:, 0] << 25) | (p[:, 1] << 5) | p[:, 2])


@pytest.mark.parametrize("when,friction", [("input", FRICTION_HST), ("input", FRICTION_DEV),
                                           ("warm", FRICTION_HST)])
def test_exact_force_pass_bit_identical(af3d, case, when, friction):
    run, (F0, T0, a0, al0) = case.forces(when, friction)
    with case.engine(af3d, af3d.FP_EXACT, when, friction, cp=run.cp) as eng:
        eng.forces()
        F, T = eng.get_forces()
        a, al = eng.get_accels()
        contacts = eng.contact_count()
    for got, want, name in ((F, F0, "F"), (T, T0, "T"), (a, a0, "a"), (al, al0, "alpha")):
        if got.tobytes() != want.tobytes():
            bad = np.nonzero(np.any(got != want, axis=1))[0]
            pytest.fail("%s differs from the oracle at %d clumps (first %d: %r vs %r)"
                        % (name, len(bad), bad[0], got[bad[0]], want[bad[0]]))
    assert contacts > case.n // 4, contacts


@pytest.mark.parametrize("when", ["input", "warm"])
def test_exact_cells_order_and_pairs(af3d, case, when):
    run, _ = case.forces(when)
    _, pp, _, _ = case.state(when)
    ids_ref, cells_ref = _sorted_slots(run)
    assert len(ids_ref) == case.n
    with case.engine(af3d, af3d.FP_EXACT, when, cp=run.cp) as eng:
        eng.forces()
        cell_of_id, ids = eng.get_cells()
        assert np.array_equal(ids, ids_ref), "(cell, id) order"
        assert np.array_equal(cell_of_id[ids_ref], cells_ref), "cell index of every clump"
        for active in (False, True):
            got = _pair_keys(eng.contact_pairs(active=active))
            want = _pair_keys(case.o.contact_pairs(run.cell_vec, run.nocup, pp, run.sys, run.cp, active=active))
            assert len(np.unique(got)) == len(got), "a pair listed twice"
            assert np.array_equal(got, want), (active, len(got), len(want))
            assert len(want) > case.n // 4


def test_fast_force_pass_within_tolerance(af3d, case):
    run, (F0, T0, a0, al0) = case.forces("warm")
    with case.engine(af3d, af3d.FP_FAST, "warm", cp=run.cp) as eng:
        eng.forces()
        F, T = eng.get_forces()
        a, al = eng.get_accels()
        pairs = {active: _pair_keys(eng.contact_pairs(active=active)) for active in (False, True)}
    errs = {"F": _rel_err(F, F0), "T": _rel_err(T, T0), "a": _rel_err(a, a0), "alpha": _rel_err(al, al0)}
    if max(errs.values()) > FORCE_RTOL:
        norm = np.linalg.norm(F0, axis=1)
        rel = np.linalg.norm(F - F0, axis=1) / np.maximum(norm, 1e-6 * norm.max())
        i = int(np.argmax(rel))
        pytest.fail("%r; worst clump %d: |F| %.3e, |dF| %.3e, max |F| %.3e, %d clumps above the bar"
                    % (errs, i, norm[i], np.linalg.norm(F[i] - F0[i]), norm.max(), int(np.sum(rel > FORCE_RTOL))))
    with case.engine(af3d, af3d.FP_EXACT, "warm", cp=run.cp) as eng:
        eng.forces()
        for active in (False, True):
            assert np.array_equal(pairs[active], _pair_keys(eng.contact_pairs(active=active))), active


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_fused_trajectory(af3d, case, mode):
    want, acc_want = case.trajectory()
    with case.engine(af3d, af3d.FP_EXACT if mode == "exact" else af3d.FP_FAST) as eng:
        eng.step(STEPS)
        p, acc, _ = eng.export_particles()
    for f in ("rr", "vv", "ww", "Rmatx", "Rmaty", "Rmatz", "rr_s"):
        scale = max(1.0, float(np.max(np.abs(want[f]))))
        err = float(np.max(np.abs(p[f] - want[f]))) / scale
        assert err <= TRAJ_RTOL, "%s: max rel error %.3e" % (f, err)
    scale = max(1.0, float(np.max(np.abs(acc_want))))
    assert float(np.max(np.abs(acc - acc_want))) / scale <= TRAJ_RTOL
