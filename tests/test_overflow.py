"""The fused force pass's fallback for clumps whose contact item lists overflow, against the
oracle.

A clump's contacts normally run from its item list: at most 32 items (boundary and sphere-pair
items), built from at most 24 partners that pass the FP32 centre test.  A clump with more runs
alone after its block's pooled items, by the per-clump cell walk (one walk per sph_id, the order
of force_part.cu:88-106's sixteen launches), with the same summation order.  These states force
that path:

  * pile:  five clumps piled almost on one spot inside a dense packing, so one clump has more
           than 32 overlapping sphere pairs (the item cap);
  * crowd: forty clumps crowded within one clump's bounding radius, so a clump has more than 24
           partners that pass the centre test (the partner cap);
  * poly:  the pile in a polydisperse packing (size factors in (0.8, 1.2]).

Bars as for every force pass: F, T, a and alpha bit-identical to the oracle in exact FP64 mode,
within 1e-10 relative per clump in fast mode; the engine's overflow counter shows that the
fallback ran; and 10 fused steps through it stay within 1e-8 of the oracle.
"""
import numpy as np
import pytest

from oracle.pyoracle import (FRICTION_DEV, FRICTION_HST, PHASE_AVALANCHE, OracleRun, dense_state, mass_inertia,
                             rotate_slope, sphere_centres)
from tests.states import flume_system

pytestmark = pytest.mark.gpu

NTAGS = 128
FORCE_RTOL = 1e-10
TRAJ_RTOL = 1e-8
N = 600


@pytest.fixture(scope="module")
def af3d():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    af3d.lib()
    return af3d


def _state(kind):
    poly = kind == "poly"
    sys, fun = flume_system(N, rmin=0.08 if poly else 0.1, rmax=0.12 if poly else 0.1, time=0.001)
    pp = dense_state(N, 31, sys, box=(1.0, 8.0, 26.0), polydisperse=1.0 / 3.0 if poly else 0.0)
    rmax = float(sys["rmax"])
    rng = np.random.default_rng(37)
    i0 = N // 2
    if kind in ("pile", "poly"):
        others = np.arange(i0 + 1, i0 + 5)
        pp["rr"][others] = pp["rr"][i0] + (rng.random((len(others), 3)) - 0.5) * 0.6 * rmax
    else:
        others = np.arange(i0 + 1, i0 + 41)
        u = rng.standard_normal((len(others), 3))
        u /= np.linalg.norm(u, axis=1)[:, None]
        pp["rr"][others] = pp["rr"][i0] + u * (rng.random(len(others))[:, None] ** (1 / 3) * 1.5 * rmax)
    mass_inertia(pp)
    sphere_centres(pp)
    rotate_slope(pp, sys)
    sys["tot_mass"] = float(pp["mass"].sum())
    return sys, fun, pp


def _rel_err(got, want):
    norm = np.linalg.norm(want, axis=1)
    floor = 1e-6 * max(float(norm.max()), 1e-300)
    return float(np.max(np.linalg.norm(got - want, axis=1) / np.maximum(norm, floor)))


@pytest.mark.parametrize("kind", ["pile", "crowd", "poly"])
@pytest.mark.parametrize("friction", [FRICTION_HST, FRICTION_DEV])
def test_overflowed_force_pass(af3d, oracle, kind, friction):
    sys, fun, pp = _state(kind)
    run = OracleRun(oracle, sys, fun, pp, ntags=NTAGS)
    assert run.forces(PHASE_AVALANCHE, friction) == 0
    want = (run.bufs["F"], run.bufs["T"]) + run.acc_f
    for mode in (af3d.FP_EXACT, af3d.FP_FAST):
        with af3d.Engine(sys, fun, ntags=NTAGS, friction=friction, fp_mode=mode) as eng:
            eng.set_grid(run.cp)
            eng.import_particles(pp)
            eng.list_overflows()
            eng.forces()
            overflows = eng.list_overflows()
            got = eng.get_forces() + eng.get_accels()
        assert overflows > 0, "the fallback did not run"
        for g, w, name in zip(got, want, ("F", "T", "a", "alpha")):
            if mode == af3d.FP_EXACT:
                assert g.tobytes() == w.tobytes(), "%s: max |diff| %.3e" % (name, np.max(np.abs(g - w)))
            else:
                assert _rel_err(g, w) <= FORCE_RTOL, (name, _rel_err(g, w))


@pytest.mark.parametrize("kind", ["pile", "crowd"])
def test_overflowed_trajectory(af3d, oracle, kind):
    sys, fun, pp = _state(kind)
    run = OracleRun(oracle, sys, fun, pp, ntags=NTAGS)
    assert run.seed_accel() == 0
    a0, al0 = [x.copy() for x in run.acc_i]
    assert run.step(10, cc0=0) == 0
    for mode in (af3d.FP_EXACT, af3d.FP_FAST):
        with af3d.Engine(sys, fun, ntags=NTAGS, fp_mode=mode) as eng:
            eng.import_particles(pp, a0, al0)
            eng.list_overflows()
            eng.step(10)
            assert eng.list_overflows() > 0
            p, a, _ = eng.export_particles()
        for f in ("rr", "vv", "ww", "Rmatx", "Rmaty", "Rmatz", "rr_s"):
            scale = max(1.0, float(np.max(np.abs(run.pp[f]))))
            err = float(np.max(np.abs(p[f] - run.pp[f]))) / scale
            assert err <= TRAJ_RTOL, (mode, f, err)
