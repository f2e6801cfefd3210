"""The permutation interval (af3d_set_resort_every) and its autotuner (af3d_autotune): the
trajectory is bit-identical whatever the interval, in both FP64 modes, so the tuner's own steps
are ordinary steps of the run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def af3d():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    af3d.lib()
    return af3d


def _state(n=600):
    from tests.states import flume_system, wall_state
    sys, fun = flume_system(n)
    return sys, fun, wall_state(n, 77, sys)


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_trajectory_does_not_depend_on_the_interval(af3d, mode):
    sys, fun, pp = _state()
    fp = af3d.FP_EXACT if mode == "exact" else af3d.FP_FAST
    outs = []
    for every in (2, 16, 64, 256):
        with af3d.Engine(sys, fun, fp_mode=fp) as e:
            e.set_resort_every(every)
            e.import_particles(pp)
            e.step(301)
            outs.append(e.export_particles())
    for o in outs[1:]:
        for x, y in zip(o, outs[0]):
            assert x.tobytes() == y.tobytes()


def test_autotune_steps_are_steps_of_the_run(af3d):
    # the tuner runs at least 3 periods of each interval (1,488 steps): a settled bed layer
    from avalancheflume3d_gb300.workloads import flume_2k, flume_state
    sys, fun, pp = flume_state(flume_2k(layout="bed"))
    with af3d.Engine(sys, fun) as a:
        a.import_particles(pp)
        t0 = float(a.get_system()["time"])
        chosen = a.autotune(32)
        assert chosen in (16, 32, 64, 128, 256)
        k = int(round((float(a.get_system()["time"]) - t0) / float(sys["dt"])))
        a.step(50)
        tuned = a.export_particles()
    with af3d.Engine(sys, fun) as b:
        b.import_particles(pp)
        b.step(k + 50)
        plain = b.export_particles()
    for x, y in zip(tuned, plain):
        assert x.tobytes() == y.tobytes()


def test_interval_argument_checks(af3d):
    sys, fun, pp = _state(100)
    with af3d.Engine(sys, fun) as e:
        for bad in (0, 1, 3, 5000):
            with pytest.raises(af3d.EngineError):
                e.set_resort_every(bad)


def test_prepare_steps_changes_nothing(af3d):
    """af3d_prepare_steps captures graphs without running them: the state is untouched and the
    steps that follow give the same bytes as steps that capture as they go."""
    sys, fun, pp = _state()
    with af3d.Engine(sys, fun) as a, af3d.Engine(sys, fun) as b:
        for e in (a, b):
            e.import_particles(pp)
            e.step(5)
        before = a.export_particles()
        a.prepare_steps(150)
        for x, y in zip(a.export_particles(), before):
            assert x.tobytes() == y.tobytes()
        a.step(150)
        b.step(150)
        for x, y in zip(a.export_particles(), b.export_particles()):
            assert x.tobytes() == y.tobytes()
