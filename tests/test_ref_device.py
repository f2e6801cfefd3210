"""The engine against the reference's OWN device kernels (``*_dev``, built from the reference's
sources into oracle/_ref/dev and driven in avalanche_dev.cu:636-693's sequence by
oracle/ref_dev.py) on the same GPU: the same state stepped by both agrees to rounding.

The reference's device twin differs from its host routines in ways the engine reproduces or
bounds: its friction is the DEV variant (``force_part.cu:487``, ``|| xi == 0``), so the engine
runs FRICTION_DEV; its build contracts multiply-adds (nvcc's default) and uses ``norm3d``
(``force_part.cu:459``); and its cell binning is an atomicAdd race (``cells.cu:150-202``), so each
clump's contacts are summed in a run-dependent order.  None of these is bit-exact, so the bar is
a tolerance: after 20 steps, positions to 1e-12 of the clump radius and velocities to 1e-9 of
the largest speed.

cell_locate_dev checks no bounds, so every step is checked before its launch (every binned
clump at least a quarter cell inside the grid and no cell more than half full), and so is the
state the engine reaches over the same steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 600
STEPS = 20


@pytest.fixture(scope="module")
def ref_dev():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import ref_dev
    if not ref_dev.available():
        pytest.skip("reference device kernels not built (the reference tree was absent at build time)")
    return ref_dev


def _state():
    from tests.states import flume_system, wall_state
    sys, fun = flume_system(N)
    pp = wall_state(N, 77, sys)
    return sys, fun, pp


def test_engine_matches_reference_device_kernels(ref_dev, oracle):
    import avalancheflume3d_gb300 as af3d
    from oracle.pyoracle import grid_for
    sys, fun, pp = _state()
    cp = grid_for(pp, sys, 16, oracle)
    zeros = np.zeros((N, 3))
    with af3d.Engine(sys, fun, friction=af3d.FRICTION_DEV) as eng:
        eng.import_particles(pp, zeros, zeros)
        eng.step(STEPS)
        mine = eng.export_particles(with_accel=False)
    sys_end = sys.copy()
    sys_end["time"] = float(sys["time"]) + STEPS * float(sys["dt"])
    for st, s in ((pp, sys), (mine, sys_end)):
        assert ref_dev.grid_margin(st, cp, s) >= 0.25
        assert 2 * ref_dev.max_occupancy(st, cp, s) <= int(cp["ntags"])
    run = ref_dev.RefDeviceRun(sys, fun, cp, pp, min_margin=0.25)
    try:
        run.set_accel(zeros, zeros)
        run.step_checked(STEPS)
        theirs, _, _ = run.export()
    finally:
        run.close()
    assert run.launches == 31 * STEPS
    rad = float(sys["rmax"])
    dr = np.abs(mine["rr"] - theirs["rr"]).max()
    vmax = float(np.abs(theirs["vv"]).max())
    dv = np.abs(mine["vv"] - theirs["vv"]).max()
    dw = np.abs(mine["ww"] - theirs["ww"]).max()
    wmax = float(np.abs(theirs["ww"]).max())
    moved = float(np.abs(theirs["rr"] - pp["rr"]).max())
    assert moved > 1e3 * dr   # the runs did move the clumps
    assert dr <= 1e-12 * rad, (dr, dv, dw)
    assert dv <= 1e-9 * vmax, (dr, dv, dw)
    assert dw <= 1e-9 * wmax, (dr, dv, dw)


def test_engine_matches_reference_device_kernels_full_workload(ref_dev, oracle):
    """The same comparison on the benchmark workload itself (262,144 clumps in a dense bed layer,
    ~2.6e5 sphere contacts per step), 10 steps."""
    import avalancheflume3d_gb300 as af3d
    from avalancheflume3d_gb300.workloads import flume_262k, flume_state
    from oracle.pyoracle import grid_for
    steps = 10
    sys, fun, pp = flume_state(flume_262k(n=262144, layout="bed"))
    n = len(pp)
    cp = grid_for(pp, sys, 16, oracle)
    zeros = np.zeros((n, 3))
    with af3d.Engine(sys, fun, friction=af3d.FRICTION_DEV) as eng:
        eng.import_particles(pp, zeros, zeros)
        eng.step(steps)
        mine = eng.export_particles(with_accel=False)
    run = ref_dev.RefDeviceRun(sys, fun, cp, pp)
    try:
        run.set_accel(zeros, zeros)
        run.step_checked(steps)
        theirs, _, _ = run.export()
    finally:
        run.close()
    rad = float(sys["rmax"])
    dr = np.abs(mine["rr"] - theirs["rr"]).max()
    dv = np.abs(mine["vv"] - theirs["vv"]).max()
    dw = np.abs(mine["ww"] - theirs["ww"]).max()
    vmax, wmax = float(np.abs(theirs["vv"]).max()), float(np.abs(theirs["ww"]).max())
    assert float(np.abs(theirs["rr"] - pp["rr"]).max()) > 1e3 * dr
    assert dr <= 1e-12 * rad, (dr, dv, dw)
    assert dv <= 1e-9 * vmax, (dr, dv, dw)
    assert dw <= 1e-9 * wmax, (dr, dv, dw)
