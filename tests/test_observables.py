"""Long runs judged on observables: granular flow is chaotic, so after a few hundred steps
single trajectories of the engine and of the oracle part ways; what must agree are the flow's
statistics.  16 seeds of a dense layer on the bed of the 40 cm x 4 cm flume, 3000 steps each, in
both FP64 modes; per seed the runout (the 95th percentile of the downslope position), the
deposit centroid (mass-weighted mean downslope position) and the mean downslope velocity, each
measured as its change since the start.  The seed-averaged changes must agree with the oracle's
within 2%.  The oracle runs in a spawn process pool, one seed per process."""
import multiprocessing as mp
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEEDS = 16
N = 1200
STEPS = 3000


def _state(seed):
    from avalancheflume3d_gb300.workloads import flume_2k, flume_state
    return flume_state(flume_2k(n=N, layout="bed", seed=seed, tilt_deg=32.0))


def _observables(pp, sys, mass):
    c, s = float(sys["cost"]), float(sys["sint"])
    x = pp["rr"][:, 0] * c - pp["rr"][:, 2] * s
    v = pp["vv"][:, 0] * c - pp["vv"][:, 2] * s
    return np.array([np.percentile(x, 95), float((mass * x).sum() / mass.sum()), float(v.mean())])


def _oracle_seed(seed):
    import sys as _sys
    _sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle.pyoracle import Oracle, OracleRun
    sys, fun, pp = _state(seed)
    o = Oracle()
    o.set_threads(1)
    run = OracleRun(o, sys, fun, pp)
    assert run.seed_accel() == 0
    before = _observables(run.pp, run.sys, run.pp["mass"])
    assert run.step(STEPS, cc0=0) == 0
    return _observables(run.pp, run.sys, run.pp["mass"]) - before


@pytest.fixture(scope="module")
def oracle_changes():
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(SEEDS, os.cpu_count() or 1)) as pool:
        return np.array(pool.map(_oracle_seed, range(1, SEEDS + 1)))


@pytest.mark.parametrize("mode", [0, 1])
def test_observables_16_seeds(oracle_changes, mode):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    got = []
    for seed in range(1, SEEDS + 1):
        sys, fun, pp = _state(seed)
        with af3d.Engine(sys, fun, fp_mode=mode) as eng:
            eng.import_particles(pp)
            eng.forces()
            eng.swap_accel()
            p0 = eng.export_particles(with_accel=False)
            before = _observables(p0, sys, p0["mass"])
            eng.step(STEPS)
            p1 = eng.export_particles(with_accel=False)
            got.append(_observables(p1, sys, p1["mass"]) - before)
    got, want = np.array(got).mean(0), oracle_changes.mean(0)
    assert np.all(np.abs(want) > 0)
    rel = np.abs(got - want) / np.abs(want)
    assert np.all(rel <= 0.02), (got, want, rel)
