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


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_results_do_not_depend_on_the_force_block(af3d, mode, oracle):
    """The fused force kernel's block (64, 96, 128 or 192 clumps pooling their contact items) changes
    no bit: one force pass (and, in exact mode, the oracle's) and 120 steps, single flume and a
    three-flume ensemble."""
    from oracle.pyoracle import OracleRun
    from tests.states import flume_system, wall_state
    fp = af3d.FP_EXACT if mode == "exact" else af3d.FP_FAST
    sys, fun, pp = _state()
    run = OracleRun(oracle, sys, fun, pp)
    assert run.forces() == 0
    outs = []
    for block in (128, 96, 64, 192):
        with af3d.Engine(sys, fun, fp_mode=fp) as e:
            e.set_force_block(block)
            assert e.force_block() == block
            e.set_grid(run.cp)
            e.import_particles(pp)
            e.forces()
            F = e.get_forces()
            if mode == "exact":
                assert F[0].tobytes() == run.bufs["F"].tobytes()
            e.swap_accel()
            e.step(120)
            outs.append((F, e.export_particles()))
    for F, o in outs[1:]:
        for x, y in zip(F + o, outs[0][0] + outs[0][1]):
            assert x.tobytes() == y.tobytes()
    specs = [(300, 35.0, 41), (180, 30.0, 42), (240, 40.0, 43)]
    flumes = []
    for n, tilt, seed in specs:
        s, f = flume_system(n, tilt=tilt)
        flumes.append((s, f, wall_state(n, seed, s)))
    ens = []
    for block in (128, 96, 64, 192):
        with af3d.Engine(np.stack([x[0] for x in flumes]), np.stack([x[1] for x in flumes]), fp_mode=fp) as e:
            e.set_force_block(block)
            e.import_particles(np.concatenate([x[2] for x in flumes]))
            e.step(60)
            ens.append(e.export_particles())
    for o in ens[1:]:
        for x, y in zip(o, ens[0]):
            assert x.tobytes() == y.tobytes()


def test_force_block_default_and_checks(af3d):
    """A new context starts with the block whose last wave of blocks is fullest on this device
    (the rule of force_shape_for, over 64, 96 and 128), and only 64, 96, 128 and 192 are
    accepted."""
    import math
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    sys, fun, pp = _state(100)

    def rule(n):
        best, best_fill = 128, -1.0
        for block, minb in ((128, 5), (96, 6), (64, 10)):
            blocks = -(-n // block)
            waves = blocks / (sms * minb)
            fill = waves / math.ceil(waves) if waves >= 1 else min(blocks, sms) / sms
            if fill > best_fill + 1e-9:
                best, best_fill = block, fill
        return best

    for n in (100, 2048, 262144, 524288):
        s = sys.copy()
        s["npart"] = n
        with af3d.Engine(s, fun) as e:
            assert e.force_block() == rule(n), n
            e.set_force_block(192)
            assert e.force_block() == 192
            for bad in (0, 32, 100, 256):
                with pytest.raises(af3d.EngineError):
                    e.set_force_block(bad)


def test_autotune_shapes_steps_are_steps_of_the_run(af3d):
    from avalancheflume3d_gb300.workloads import flume_2k, flume_state
    sys, fun, pp = flume_state(flume_2k(layout="bed"))
    with af3d.Engine(sys, fun, fp_mode=af3d.FP_FAST) as a:
        a.import_particles(pp)
        t0 = float(a.get_system()["time"])
        timings = {}
        every, block = a.autotune_shapes(32, timings)
        assert every in (16, 32, 64, 128, 256) and block in (64, 96, 128, 192)
        assert a.force_block() == block
        assert set(timings["block"]) == {64, 96, 128, 192} and all(v > 0 for v in timings["block"].values())
        k = int(round((float(a.get_system()["time"]) - t0) / float(sys["dt"])))
        a.step(50)
        tuned = a.export_particles()
    with af3d.Engine(sys, fun, fp_mode=af3d.FP_FAST) as b:
        b.import_particles(pp)
        b.step(k + 50)
        plain = b.export_particles()
    for x, y in zip(tuned, plain):
        assert x.tobytes() == y.tobytes()
