"""Long runs judged on observables: granular flow is chaotic, so after a few hundred steps
single trajectories of the engine and of the oracle part ways; what must agree are the flow's
statistics.  16 seeds of a dense layer on the bed of the 40 cm x 4 cm flume, 3000 steps each, in
both FP64 modes; per seed the runout (the 95th percentile of the downslope position), the
deposit centroid (mass-weighted mean downslope position) and the mean downslope velocity, each
measured as its change since the start.  The seed-averaged changes must agree with the oracle's
within 2%.  The oracle runs in a spawn process pool, one seed per process.  The same check at the
2,048-clump flume's full 50,000-step horizon compares with the oracle's committed observables."""
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


# The 2,048-clump flume over its full 50,000-step horizon (0.1 s), 16 seeds, against the oracle's
# observables committed in tests/golden/observables_flume2k.npz (tests/golden/make_observables.py:
# single-threaded oracle runs of about 10 minutes each).  The 16 seeds run on the GPU as one
# batched ensemble, whose flumes evolve exactly as they do alone.
@pytest.fixture(scope="module")
def flume2k_golden():
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "observables_flume2k.npz")
    with np.load(path) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("layout", ["lattice", "bed"])
def test_observables_flume2k_full_horizon(flume2k_golden, layout, mode):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    from avalancheflume3d_gb300.workloads import ensemble_state, flume_2k
    g = flume2k_golden
    li = list(g["layouts"]).index(layout)
    seeds = [int(s) for s in g["seeds"]]
    sys, fun, pp = ensemble_state([flume_2k(layout=layout, seed=s) for s in seeds])
    with af3d.Engine(sys, fun, fp_mode=mode) as eng:
        eng.import_particles(pp)
        eng.forces()
        eng.swap_accel()
        eng.step(int(g["steps"]))
        assert eng.status() == 0
        p1 = eng.export_particles(with_accel=False)
        spans = [eng.flume_slice(f) for f in range(len(seeds))]
    before = np.array([_observables(pp[s], sys[f], pp["mass"][s]) for f, s in enumerate(spans)])
    after = np.array([_observables(p1[s], sys[f], p1["mass"][s]) for f, s in enumerate(spans)])
    # the same initial states as the oracle's (generated by the same host routines)
    np.testing.assert_allclose(before, g["before"][li], rtol=1e-9, atol=1e-12)
    got = (after - before).mean(0)
    want = (g["after"][li] - g["before"][li]).mean(0)
    assert np.all(np.abs(want) > 0)
    rel = np.abs(got - want) / np.abs(want)
    print("flume2k %s mode %d: relative differences (runout, centroid, velocity)" % (layout, mode), rel)
    assert np.all(rel <= 0.02), (layout, mode, got, want, rel)
