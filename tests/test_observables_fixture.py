"""The committed long-run observables (tests/golden/observables_flume2k.npz, written by
tests/golden/make_observables.py from 50,000-step oracle runs) belong to the initial states the
workload builders make today: the runout, deposit centroid and mean velocity of every seed's
input state, recomputed here, equal the fixture's starting values.  A change to the builders
that would leave the fixture stale fails here, on the CPU, before any GPU run compares against
it."""
import os

import numpy as np

from tests.golden.make_observables import LAYOUTS, SEEDS, STEPS, observables

HERE = os.path.dirname(os.path.abspath(__file__))


def test_fixture_matches_the_workload_builders():
    from avalancheflume3d_gb300.workloads import flume_2k, flume_state
    with np.load(os.path.join(HERE, "golden", "observables_flume2k.npz")) as z:
        assert tuple(z["layouts"]) == LAYOUTS and tuple(int(s) for s in z["seeds"]) == SEEDS
        assert int(z["steps"]) == STEPS
        before, after = z["before"], z["after"]
    assert before.shape == after.shape == (len(LAYOUTS), len(SEEDS), 3)
    for li, layout in enumerate(LAYOUTS):
        for si, seed in enumerate(SEEDS):
            sys_, _, pp = flume_state(flume_2k(layout=layout, seed=seed))
            np.testing.assert_allclose(observables(pp, sys_), before[li, si], rtol=1e-12, atol=1e-12)
    # every run moved downslope: the observables changed
    assert np.all(np.abs(after - before).mean(axis=1) > 0)
