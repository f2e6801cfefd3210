"""af3d_step_host -- import, one step and export in one call, the export of each quarter of the
clumps overlapping the force pass of the next -- against the three calls it replaces
(af3d_import_particles, af3d_step(1), af3d_export_particles) on a second context from the same
state: the exported particles and accelerations are byte-identical, call after call, in both
FP64 modes, for clump counts that split into uneven parts or into one, with in == out."""
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


def _state(n, seed=77):
    from tests.states import flume_system, wall_state
    sys, fun = flume_system(n)
    return sys, fun, wall_state(n, seed, sys)


@pytest.mark.parametrize("n,mode", [(600, "exact"), (600, "fast"), (100, "exact"), (2053, "exact")])
def test_step_host_equals_import_step_export(af3d, n, mode):
    sys, fun, pp0 = _state(n)
    fp = af3d.FP_EXACT if mode == "exact" else af3d.FP_FAST
    rng = np.random.default_rng(3)
    acc0, anga0 = rng.standard_normal((n, 3)) * 10.0, rng.standard_normal((n, 3))
    with af3d.Engine(sys, fun, fp_mode=fp) as a, af3d.Engine(sys, fun, fp_mode=fp) as b:
        # both contexts first take a few ordinary steps (b's slots then follow a cell permutation)
        for e in (a, b):
            e.import_particles(pp0, acc0, anga0)
            e.step(3)
        pa, aa, la = a.export_particles()
        pb, ab, lb = pa.copy(), aa.copy(), la.copy()
        for _ in range(3):
            # the three calls
            a.import_particles(pa, aa, la)
            a.step(1)
            pa, aa, la = a.export_particles()
            # the fused call, in place
            b.step_host(pb, ab, lb, acc_out=ab, anga_out=lb)
            assert pb.tobytes() == pa.tobytes()
            assert ab.tobytes() == aa.tobytes()
            assert lb.tobytes() == la.tobytes()
        # the context is left in a state ordinary steps continue from
        a.step(2)
        b.step(2)
        assert b.export_particles(with_accel=False).tobytes() == a.export_particles(with_accel=False).tobytes()


def test_step_host_without_accelerations(af3d):
    sys, fun, pp0 = _state(600)
    with af3d.Engine(sys, fun) as a, af3d.Engine(sys, fun) as b:
        a.import_particles(pp0)
        a.step(1)
        want = a.export_particles(with_accel=False)
        out = np.zeros_like(pp0)
        b.step_host(pp0, out=out)
        assert out.tobytes() == want.tobytes()


def test_step_host_on_an_ensemble(af3d):
    """Two flumes back to back in one context: the fused call matches the three calls."""
    from tests.states import flume_system, wall_state
    syss, funs, pps = [], [], []
    for k, m in enumerate((300, 220)):
        s, f = flume_system(m, mu_pp=0.3 + 0.2 * k)
        syss.append(s)
        funs.append(f)
        pps.append(wall_state(m, 20 + k, s))
    sys, fun, pp0 = np.stack(syss), np.stack(funs), np.concatenate(pps)
    with af3d.Engine(sys, fun) as a, af3d.Engine(sys, fun) as b:
        for e in (a, b):
            e.import_particles(pp0)
            e.step(2)
        pa = a.export_particles(with_accel=False)
        pb = pa.copy()
        for _ in range(2):
            a.import_particles(pa)
            a.step(1)
            pa = a.export_particles(with_accel=False)
            b.step_host(pb)
            assert pb.tobytes() == pa.tobytes()
