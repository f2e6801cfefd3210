"""Polydisperse clumps: every clump scaled by its own factor in [0.8, 1.2] (sphere radius and
tetrahedron edge together, mass and inertia from calculate_particle_parameters' formulas), as in
the 524,288-clump funnel-and-hopper configuration.  The cell size follows the largest radius.
Same bars as the monodisperse cases: one force pass bit-exact (exact mode) or within 1e-10
(fast mode); 100-step trajectories within 1e-8."""
import numpy as np
import pytest

from oracle.pyoracle import (FRICTION_HST, PHASE_AVALANCHE, PHASE_FILL, OracleRun, dense_state, mass_inertia,
                             rotate_slope, sphere_centres)
from tests.states import flume_system, wall_state

pytestmark = pytest.mark.gpu

R_NOM = 0.1


@pytest.fixture(scope="module")
def af3d():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    af3d.lib()
    return af3d


def _state(kind, n, seed, time):
    sys, fun = flume_system(n, rmin=0.8 * R_NOM, rmax=1.2 * R_NOM, time=time)
    if kind == "dense":
        # radius = rmax * (1 - u/3), u ~ U[0, 1): a factor in (0.8, 1.2] of the nominal radius
        pp = dense_state(n, seed, sys, box=(1.0, 8.0, 26.0), polydisperse=1.0 / 3.0)
    else:
        pp = wall_state(n, seed, sys)
        rng = np.random.default_rng(seed + 1000)
        pp["radius"] = R_NOM * (0.8 + 0.4 * rng.random(n))
        mass_inertia(pp)
        sphere_centres(pp)
        rotate_slope(pp, sys)
    assert pp["radius"].min() >= 0.8 * R_NOM - 1e-15 and pp["radius"].max() <= 1.2 * R_NOM + 1e-15
    sys["tot_mass"] = float(pp["mass"].sum())
    return sys, fun, pp


def _engine(af3d, sys, fun, pp, cp, mode, phase=PHASE_AVALANCHE, acc=None, anga=None):
    eng = af3d.Engine(sys, fun, phase=phase, fp_mode=mode)
    eng.set_grid(cp)
    eng.import_particles(pp, acc, anga)
    return eng


def _rel_err(got, want):
    norm = np.linalg.norm(want, axis=1)
    floor = 1e-6 * max(float(norm.max()), 1e-300)
    return float(np.max(np.linalg.norm(got - want, axis=1) / np.maximum(norm, floor)))


@pytest.mark.parametrize("kind,phase", [("dense", PHASE_AVALANCHE), ("wall", PHASE_AVALANCHE),
                                        ("dense", PHASE_FILL)])
def test_polydisperse_force_pass(af3d, oracle, kind, phase):
    n = 900
    sys, fun, pp = _state(kind, n, 17, time=-0.5 if phase == PHASE_FILL else 0.001)
    run = OracleRun(oracle, sys, fun, pp)
    assert run.forces(phase, FRICTION_HST) == 0
    for mode in (af3d.FP_EXACT, af3d.FP_FAST):
        with _engine(af3d, sys, fun, pp, run.cp, mode, phase) as eng:
            eng.forces()
            F, T = eng.get_forces()
            a, al = eng.get_accels()
            assert eng.contact_count() > 0
        if mode == af3d.FP_EXACT:
            assert F.tobytes() == run.bufs["F"].tobytes() and T.tobytes() == run.bufs["T"].tobytes()
            assert a.tobytes() == run.acc_f[0].tobytes() and al.tobytes() == run.acc_f[1].tobytes()
        else:
            errs = [_rel_err(F, run.bufs["F"]), _rel_err(T, run.bufs["T"]), _rel_err(a, run.acc_f[0]),
                    _rel_err(al, run.acc_f[1])]
            assert max(errs) <= 1e-10, errs


@pytest.mark.parametrize("mode", [0, 1])
def test_polydisperse_trajectory_100_steps(af3d, oracle, mode):
    n = 600
    sys, fun, pp = _state("wall", n, 23, time=0.0)
    run = OracleRun(oracle, sys, fun, pp)
    assert run.seed_accel() == 0
    a0, al0 = [x.copy() for x in run.acc_i]
    with _engine(af3d, sys, fun, pp, run.cp, mode, acc=a0, anga=al0) as eng:
        eng.step(100)
        p, a, _ = eng.export_particles()
    assert run.step(100, cc0=0) == 0
    for f in ("rr", "vv", "ww", "Rmatx", "Rmaty", "Rmatz", "rr_s", "radius"):
        x, y = p[f], run.pp[f]
        scale = max(1.0, float(np.max(np.abs(y))))
        assert float(np.max(np.abs(x - y))) / scale <= 1e-8, f
