"""Golden fixtures generated from the reference's own routines (tests/golden/make_golden.py).

The CPU tests pin the oracle restatement to them on any machine (including where the reference
tree is absent); the GPU tests check the CUDA engine against them through the C ABI."""
import glob
import os

import numpy as np
import pytest

from oracle.pyoracle import Oracle, OracleRun

HERE = os.path.dirname(os.path.abspath(__file__))
# the force-pass fixtures of make_golden.py (observables_*.npz are make_observables.py's)
FIXTURES = sorted(f for f in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                  if not os.path.basename(f).startswith("observables_"))
STEP1_RTOL = 1e-13     # one step: only libm's sin/cos may differ between platforms
STEP100_RTOL = 1e-8


def load(fn):
    z = np.load(fn)
    return {k: z[k] for k in z.files}


def _same(a, b):
    return np.asarray(a).tobytes() == np.asarray(b).tobytes()


def _close(p, q, rtol):
    for f in ("rr", "vv", "ww", "Rmatx", "Rmaty", "Rmatz", "rr_s", "radius"):
        scale = max(1.0, float(np.max(np.abs(q[f]))))
        err = float(np.max(np.abs(p[f] - q[f]))) / scale
        assert err <= rtol, "%s: %.3e" % (f, err)


def test_fixtures_present():
    assert len(FIXTURES) >= 3


@pytest.mark.parametrize("fn", FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def test_oracle_reproduces_golden(fn):
    g = load(fn)
    phase = int(g["phase"])
    run = OracleRun(Oracle(), g["sys"], g["fun"], g["pp"], cp=g["cell"])
    assert run.forces(phase) == 0
    assert _same(run.bufs["F"], g["force"]) and _same(run.bufs["T"], g["torque"])
    a, al = run.acc_f
    assert _same(a, g["acc_f"]) and _same(al, g["anga_f"])
    pairs = Oracle().contact_pairs(run.cell_vec, run.nocup, run.pp, run.sys, run.cp)
    assert _same(pairs, g["pairs"])
    run2 = OracleRun(Oracle(), g["sys"], g["fun"], g["pp"], cp=g["cell"], acc=g["acc_i0"], anga=g["anga_i0"])
    run2.step(1, phase)
    _close(run2.pp, g["pp_1"], STEP1_RTOL)
    run2.step(99, phase)
    _close(run2.pp, g["pp_100"], STEP100_RTOL)
    assert float(run2.sys["time"]) == float(g["time_100"])


@pytest.mark.gpu
@pytest.mark.parametrize("fn", FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def test_engine_reproduces_golden(fn):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    g = load(fn)
    phase = int(g["phase"])
    with af3d.Engine(g["sys"], g["fun"], phase=phase) as eng:
        eng.set_grid(g["cell"])
        eng.import_particles(g["pp"])
        eng.forces()
        F, T = eng.get_forces()
        a, al = eng.get_accels()
        assert _same(F, g["force"]) and _same(T, g["torque"])
        assert _same(a, g["acc_f"]) and _same(al, g["anga_f"])
        cell_of_id, ids = eng.get_cells()
        assert np.array_equal(ids, g["sorted_ids"]) and np.array_equal(cell_of_id[ids], g["sorted_cells"])
        got = set(map(tuple, eng.contact_pairs().tolist()))
        assert got == set(map(tuple, g["pairs"].tolist()))
    with af3d.Engine(g["sys"], g["fun"], phase=phase) as eng:
        eng.set_grid(g["cell"])
        eng.import_particles(g["pp"], g["acc_i0"], g["anga_i0"])
        for k in range(100):
            eng.init_verlet()
            eng.advance_time()
            eng.rotate_vectors()
            eng.clear_forces()
            eng.cell_build()
            if phase == af3d.PHASE_FILL:
                eng.force_part(0)
                for nw in range(3):
                    eng.force_hop(nw)
            else:
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
            if k == 0:
                p1 = eng.export_particles(with_accel=False)
        p100 = eng.export_particles(with_accel=False)
    _close(p1, g["pp_1"], STEP1_RTOL)
    _close(p100, g["pp_100"], STEP100_RTOL)
