"""af3d_save_checkpoint / af3d_load_checkpoint: a run stopped half way, saved, and loaded into a
fresh context continues bit for bit as the run that did not stop -- across the device re-grid
after the first step, in both FP64 modes (the mode is restored from the file), and for an
ensemble of flumes.  A checkpoint of another context shape is refused."""
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


@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_checkpoint_continues_bit_for_bit(af3d, tmp_path, mode):
    from tests.states import flume_system, wall_state
    n = 600
    sys, fun = flume_system(n)
    pp = wall_state(n, 77, sys)
    fp = af3d.FP_EXACT if mode == "exact" else af3d.FP_FAST
    path = str(tmp_path / "run.ckpt")
    with af3d.Engine(sys, fun, fp_mode=fp) as a:
        a.import_particles(pp)
        a.forces()
        a.swap_accel()
        a.step(70)
        a.save_checkpoint(path)
        a.step(70)
        want = a.export_particles()
        want_sys = a.get_system()
    with af3d.Engine(sys, fun) as b:   # created in exact mode: the file restores the mode
        b.load_checkpoint(path)
        b.step(70)
        got = b.export_particles()
        got_sys = b.get_system()
    for x, y in zip(got, want):
        assert x.tobytes() == y.tobytes()
    assert got_sys.tobytes() == want_sys.tobytes()


def test_checkpoint_of_an_ensemble(af3d, tmp_path):
    from tests.states import flume_system, wall_state
    sizes = (300, 200)
    syss, funs, pps = [], [], []
    for k, m in enumerate(sizes):
        s, f = flume_system(m, mu_pp=0.3 + 0.2 * k)
        syss.append(s)
        funs.append(f)
        pps.append(wall_state(m, 10 + k, s))
    sys, fun, pp = np.stack(syss), np.stack(funs), np.concatenate(pps)
    path = str(tmp_path / "ens.ckpt")
    with af3d.Engine(sys, fun) as a:
        a.import_particles(pp)
        a.step(40)
        a.save_checkpoint(path)
        a.step(40)
        want = a.export_particles(with_accel=False)
    with af3d.Engine(sys, fun) as b:
        b.load_checkpoint(path)
        b.step(40)
        assert b.export_particles(with_accel=False).tobytes() == want.tobytes()
    s1, f1 = flume_system(500)
    with af3d.Engine(s1, f1) as c, pytest.raises(af3d.EngineError):
        c.load_checkpoint(path)   # one flume of 500 clumps: another shape
