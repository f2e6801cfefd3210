"""GPU parity of the CUDA engine (through the C ABI) against the pinned CPU oracle.

Bars (all on identical input states):
  * cell index of every clump, the (cell, id)-sorted order and the contact-pair sets: bit-exact
  * forces, torques and accelerations of one force pass: bit-exact (the kernels keep the
    reference's FP64 evaluation order with no contraction, and the reference's summation order)
  * trajectories over 100 steps: within 1e-8 relative (init_Verlet's sin/cos come from CUDA's
    libm, which may differ from the host libm in the last bit)
"""
import numpy as np
import pytest

from oracle.pyoracle import (FRICTION_DEV, FRICTION_HST, PHASE_AVALANCHE, PHASE_FILL, Oracle, OracleRun,
                             dense_state)
from tests.states import Work, flume_system, grid_from_state, run_forces, sorted_order, wall_state

pytestmark = pytest.mark.gpu

TRAJ_RTOL = 1e-8


@pytest.fixture(scope="module")
def af3d():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    af3d.lib()
    return af3d


def _engine(af3d, sys, fun, pp, cp, phase=PHASE_AVALANCHE, friction=FRICTION_HST, ntags=9, acc=None,
            anga=None):
    eng = af3d.Engine(sys, fun, ntags=ntags, phase=phase, friction=friction)
    eng.set_grid(cp)                 # a grid set before the import is kept (no device re-grid)
    eng.import_particles(pp, acc, anga)
    return eng


def _state(kind, n, seed, time=0.001):
    sys, fun = flume_system(n, time=time)
    if kind == "wall":
        pp = wall_state(n, seed, sys)
    else:
        pp = dense_state(n, seed, sys, box=(1.0, 8.0, 26.0))
    return sys, fun, pp


def _same(a, b):
    return np.asarray(a).tobytes() == np.asarray(b).tobytes()


def _describe(got, want):
    d = np.abs(got - want)
    i = np.unravel_index(np.argmax(d), d.shape)
    return "max |diff| %.3e at %s (got %r want %r)" % (d[i], i, got[i], want[i])


@pytest.mark.parametrize("kind,phase,friction", [
    ("wall", PHASE_AVALANCHE, FRICTION_HST),
    ("dense", PHASE_AVALANCHE, FRICTION_HST),
    ("dense", PHASE_AVALANCHE, FRICTION_DEV),
    ("dense", PHASE_FILL, FRICTION_HST),
    ("wall", PHASE_FILL, FRICTION_DEV),
])
def test_force_pass_bit_exact(af3d, oracle, kind, phase, friction):
    n = 900
    sys, fun, pp = _state(kind, n, 3, time=-0.5 if phase == PHASE_FILL else 0.001)
    run = OracleRun(oracle, sys, fun, pp)
    assert run.forces(phase, friction) == 0
    with _engine(af3d, sys, fun, pp, run.cp, phase, friction) as eng:
        eng.forces()
        F, T = eng.get_forces()
        a, al = eng.get_accels()
        contacts = eng.contact_count()
    ao, alo = run.acc_f
    assert _same(F, run.bufs["F"]), _describe(F, run.bufs["F"])
    assert _same(T, run.bufs["T"]), _describe(T, run.bufs["T"])
    assert _same(a, ao), _describe(a, ao)
    assert _same(al, alo), _describe(al, alo)
    assert contacts > 0


@pytest.mark.parametrize("kind", ["wall", "dense"])
def test_cells_and_contact_pairs_exact(af3d, oracle, kind):
    n = 900
    sys, fun, pp = _state(kind, n, 5)
    cp = grid_from_state(pp, sys, 9, oracle)
    w = Work(n, cp)
    run_forces(oracle, sys, fun, cp, pp, w, PHASE_AVALANCHE)
    ids_ref, cells_ref = sorted_order(cp, w)
    with _engine(af3d, sys, fun, pp, cp) as eng:
        eng.forces()
        cell_of_id, ids = eng.get_cells()
        assert np.array_equal(ids, ids_ref), "sorted (cell, id) order"
        assert np.array_equal(cell_of_id[ids_ref], cells_ref), "cell index of every clump"
        for active in (False, True):
            got = eng.contact_pairs(active=active)
            want = oracle.contact_pairs(w.cell_vec, w.nocup, pp, sys, cp, active=active)
            gs = set(map(tuple, got.tolist()))
            ws = set(map(tuple, want.tolist()))
            assert len(got) == len(gs) and gs == ws, (len(gs), len(ws), len(gs ^ ws))
            assert len(ws) > 0


def test_per_routine_path_equals_fused(af3d, oracle):
    """The reference's call sequence through the per-routine entry points gives the same bits as
    the fused pass and the oracle."""
    n = 700
    sys, fun, pp = _state("wall", n, 9)
    run = OracleRun(oracle, sys, fun, pp)
    assert run.forces(PHASE_AVALANCHE) == 0
    with _engine(af3d, sys, fun, pp, run.cp) as eng:
        eng.rotate_vectors()
        eng.clear_forces()
        eng.cell_build()
        for nw in range(3):
            eng.force_hop(nw)
        eng.force_funnel()
        eng.force_fcorners()
        eng.force_walls()
        for sph in range(1, 17):
            eng.force_part(sph)
        eng.force_flume()
        eng.get_accel()
        F, T = eng.get_forces()
        a, al = eng.get_accels()
    assert _same(F, run.bufs["F"]) and _same(T, run.bufs["T"])
    assert _same(a, run.acc_f[0]) and _same(al, run.acc_f[1])


def test_per_routine_step_matches_oracle_step(af3d, oracle):
    """init_Verlet ... finish_Verlet, swap through the per-routine entry points for 3 steps."""
    n = 600
    sys, fun, pp = _state("dense", n, 13, time=0.0)
    run = OracleRun(oracle, sys, fun, pp)
    assert run.seed_accel() == 0
    a0, al0 = [x.copy() for x in run.acc_i]
    with _engine(af3d, sys, fun, pp, run.cp, acc=a0, anga=al0) as eng:
        for _ in range(3):
            eng.init_verlet()
            eng.advance_time()
            eng.rotate_vectors()
            eng.clear_forces()
            eng.cell_build()
            for nw in range(3):
                eng.force_hop(nw)
            eng.force_funnel()
            eng.force_fcorners()
            eng.force_walls()
            eng.force_part(0)
            eng.force_flume()
            eng.get_accel()
            eng.finish_verlet()
            eng.swap_accel()
        p, a, al = eng.export_particles()
    assert run.step(3) == 0
    _check_traj(p, run.pp, a, run.acc_i[0])


def _check_traj(p, q, a=None, b=None, rtol=TRAJ_RTOL):
    for f in ("rr", "vv", "ww", "Rmatx", "Rmaty", "Rmatz", "rr_s", "radius"):
        x, y = p[f], q[f]
        scale = max(1.0, float(np.max(np.abs(y))))
        err = float(np.max(np.abs(x - y))) / scale
        assert err <= rtol, "%s: max rel error %.3e" % (f, err)
    if a is not None:
        scale = max(1.0, float(np.max(np.abs(b))))
        assert float(np.max(np.abs(a - b))) / scale <= rtol


@pytest.mark.parametrize("phase", [PHASE_AVALANCHE, PHASE_FILL])
def test_trajectory_100_steps(af3d, oracle, phase):
    n = 600
    sys, fun, pp = _state("dense" if phase == PHASE_FILL else "wall", n, 21,
                          time=-0.5 if phase == PHASE_FILL else 0.0)
    run = OracleRun(oracle, sys, fun, pp)
    assert run.seed_accel(phase) == 0
    a0, al0 = [x.copy() for x in run.acc_i]
    with _engine(af3d, sys, fun, pp, run.cp, phase=phase, acc=a0, anga=al0) as eng:
        eng.step(100)
        p, a, al = eng.export_particles()
        t = float(eng.get_system()["time"])
    assert run.step(100, phase, cc0=0) == 0
    assert t == float(run.sys["time"])
    _check_traj(p, run.pp, a, run.acc_i[0])


def test_step_regrid_schedule(af3d, oracle):
    """af3d_step re-grids on the device after the step with cc % 2000 == 0, like the reference."""
    n = 400
    sys, fun, pp = _state("wall", n, 2, time=0.0)
    run = OracleRun(oracle, sys, fun, pp)
    run.seed_accel()
    a0, al0 = [x.copy() for x in run.acc_i]
    with _engine(af3d, sys, fun, pp, run.cp, acc=a0, anga=al0) as eng:
        eng.step(5)
        g = eng.get_grid()
        p, a, _ = eng.export_particles()
    run.step(5, cc0=0)
    assert _same(g, run.cp), "grid derived on the device differs from cell_dim + derivation"
    _check_traj(p, run.pp, a, run.acc_i[0])


def test_device_regrid_bit_exact(af3d, oracle):
    n = 800
    sys, fun, pp = _state("wall", n, 4)
    run = OracleRun(oracle, sys, fun, pp)
    with af3d.Engine(sys, fun) as eng:
        eng.import_particles(pp)          # first import derives the grid on the device
        g = eng.get_grid()
    assert _same(g, run.cp)


def test_removed_clumps(af3d, oracle):
    n = 400
    sys, fun, pp = _state("wall", n, 5, time=0.01)
    sys["side"][0] = float(np.median(pp["rr"][:, 0]))
    run = OracleRun(oracle, sys, fun, pp)
    run.seed_accel()
    a0, al0 = [x.copy() for x in run.acc_i]
    with _engine(af3d, sys, fun, pp, run.cp, acc=a0, anga=al0) as eng:
        eng.step(6)
        p, a, al = eng.export_particles()
    run.step(6, cc0=0)
    live = run.pp["radius"] > 0
    assert np.array_equal(p["radius"] > 0, live) and (~live).sum() > n // 4
    _check_traj(p[live], run.pp[live])
    assert np.all(p["vv"][~live] == 0)


def test_capacity_and_escape_are_reported(af3d, oracle):
    n = 300
    sys, fun, pp = _state("dense", n, 6)
    cp = grid_from_state(pp, sys, 9, oracle)
    with _engine(af3d, sys, fun, pp, cp, ntags=2) as eng:       # at most one clump per cell
        with pytest.raises(af3d.EngineError) as e:
            eng.forces()
        assert e.value.code == 6
    small = cp.copy()
    small["ncell"] = np.maximum(cp["ncell"] // 2, 1)
    small["ncell3"] = int(np.prod(small["ncell"]))
    with _engine(af3d, sys, fun, pp, small) as eng:             # grid too small: clumps escape
        with pytest.raises(af3d.EngineError) as e:
            eng.forces()
        assert e.value.code == 4


def test_single_and_empty(af3d, oracle):
    from oracle.pyoracle import CELL_PAR, grid_from_bbox
    sys, fun, pp = _state("wall", 1, 7)
    # cell_dim's box around one clump is narrower than a cell: the reference derives ncell.x = 0
    # and then exits on a negative cell index; the engine refuses such a grid with an error.
    degenerate = OracleRun(oracle, sys, fun, pp).cp
    assert int(degenerate["ncell3"]) == 0
    with af3d.Engine(sys, fun) as eng:
        with pytest.raises(af3d.EngineError):
            eng.import_particles(pp)
    cp = np.zeros((), dtype=CELL_PAR)
    cp["ntags"] = 9
    cp["rr_min"], cp["rr_max"] = pp["rr"][0] - 1.0, pp["rr"][0] + 1.0
    grid_from_bbox(cp, sys)
    run = OracleRun(oracle, sys, fun, pp, cp=cp)
    assert run.forces() == 0
    with _engine(af3d, sys, fun, pp, cp) as eng:
        eng.forces()
        F, T = eng.get_forces()
    assert _same(F, run.bufs["F"]) and _same(T, run.bufs["T"])
    sys0, fun0 = flume_system(0)
    with af3d.Engine(sys0, fun0) as eng:
        eng.import_particles(np.zeros(0, dtype=af3d.PARTICLE))
        eng.set_grid(cp)
        eng.step(2)


def test_determinism(af3d, oracle):
    n = 3000
    sys, fun, pp = _state("dense", n, 8, time=0.0)
    run = OracleRun(oracle, sys, fun, pp)
    outs = []
    for _ in range(2):
        with _engine(af3d, sys, fun, pp, run.cp) as eng:
            eng.forces()
            eng.swap_accel()
            eng.step(30)
            outs.append(eng.export_particles())
    assert _same(outs[0][0], outs[1][0]) and _same(outs[0][1], outs[1][1])
