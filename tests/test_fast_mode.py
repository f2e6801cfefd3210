"""Fast FP64 mode (AF3D_FP_FAST: contracted multiply-adds, reciprocal-square-root normals)
against the pinned CPU oracle, at the tolerances the path is specified to:

  * one force pass on an identical input state: forces, torques and accelerations within 1e-10
    relative, per clump, of the oracle (relative to the clump's vector norm; a clump whose net
    force nearly cancels is measured against 1e-6 of the largest norm in the state instead)
  * trajectories over 100 steps within 1e-8 relative (the exact mode's bar as well)
  * cell indices, sorted order and contact-pair sets: identical to the exact mode (they depend
    on positions only)
"""
import numpy as np
import pytest

from oracle.pyoracle import FRICTION_DEV, FRICTION_HST, PHASE_AVALANCHE, PHASE_FILL, OracleRun, dense_state
from tests.states import flume_system, wall_state

pytestmark = pytest.mark.gpu

FORCE_RTOL = 1e-10
TRAJ_RTOL = 1e-8


@pytest.fixture(scope="module")
def af3d():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    af3d.lib()
    return af3d


def _state(kind, n, seed, time=0.001):
    sys, fun = flume_system(n, time=time)
    pp = wall_state(n, seed, sys) if kind == "wall" else dense_state(n, seed, sys, box=(1.0, 8.0, 26.0))
    return sys, fun, pp


def _engine(af3d, sys, fun, pp, cp, mode, phase=PHASE_AVALANCHE, friction=FRICTION_HST, acc=None, anga=None):
    eng = af3d.Engine(sys, fun, phase=phase, friction=friction, fp_mode=mode)
    eng.set_grid(cp)
    eng.import_particles(pp, acc, anga)
    return eng


def _rel_err(got, want):
    """Per-clump |got - want| / max(|want|, 1e-6 max|want|), maximised over clumps."""
    norm = np.linalg.norm(want, axis=1)
    floor = 1e-6 * max(float(norm.max()), 1e-300)
    return float(np.max(np.linalg.norm(got - want, axis=1) / np.maximum(norm, floor)))


@pytest.mark.parametrize("kind,phase,friction", [
    ("wall", PHASE_AVALANCHE, FRICTION_HST),
    ("dense", PHASE_AVALANCHE, FRICTION_HST),
    ("dense", PHASE_AVALANCHE, FRICTION_DEV),
    ("dense", PHASE_FILL, FRICTION_HST),
    ("wall", PHASE_FILL, FRICTION_DEV),
])
def test_fast_force_pass_within_tolerance(af3d, oracle, kind, phase, friction):
    n = 900
    sys, fun, pp = _state(kind, n, 3, time=-0.5 if phase == PHASE_FILL else 0.001)
    run = OracleRun(oracle, sys, fun, pp)
    assert run.forces(phase, friction) == 0
    with _engine(af3d, sys, fun, pp, run.cp, af3d.FP_FAST, phase, friction) as eng:
        eng.forces()
        F, T = eng.get_forces()
        a, al = eng.get_accels()
        contacts = eng.contact_count()
    ao, alo = run.acc_f
    errs = {"F": _rel_err(F, run.bufs["F"]), "T": _rel_err(T, run.bufs["T"]), "a": _rel_err(a, ao),
            "alpha": _rel_err(al, alo)}
    assert max(errs.values()) <= FORCE_RTOL, errs
    assert contacts > 0


def test_fast_differs_from_exact_only_in_rounding(af3d, oracle):
    """The fast pass is a different evaluation of the same law: not bit-identical in general,
    but within a few ulps (this also shows that the fast kernels actually ran)."""
    n = 900
    sys, fun, pp = _state("dense", n, 11)
    run = OracleRun(oracle, sys, fun, pp)
    assert run.forces() == 0
    out = {}
    for mode in (af3d.FP_EXACT, af3d.FP_FAST):
        with _engine(af3d, sys, fun, pp, run.cp, mode) as eng:
            eng.forces()
            out[mode] = eng.get_forces()[0]
    assert out[af3d.FP_EXACT].tobytes() == run.bufs["F"].tobytes()
    assert out[af3d.FP_FAST].tobytes() != out[af3d.FP_EXACT].tobytes()
    assert _rel_err(out[af3d.FP_FAST], out[af3d.FP_EXACT]) <= FORCE_RTOL


@pytest.mark.parametrize("phase", [PHASE_AVALANCHE, PHASE_FILL])
def test_fast_trajectory_100_steps(af3d, oracle, phase):
    n = 600
    sys, fun, pp = _state("dense" if phase == PHASE_FILL else "wall", n, 21,
                          time=-0.5 if phase == PHASE_FILL else 0.0)
    run = OracleRun(oracle, sys, fun, pp)
    assert run.seed_accel(phase) == 0
    a0, al0 = [x.copy() for x in run.acc_i]
    with _engine(af3d, sys, fun, pp, run.cp, af3d.FP_FAST, phase=phase, acc=a0, anga=al0) as eng:
        eng.step(100)
        p, a, _ = eng.export_particles()
    assert run.step(100, phase, cc0=0) == 0
    for f in ("rr", "vv", "ww", "Rmatx", "Rmaty", "Rmatz", "rr_s"):
        x, y = p[f], run.pp[f]
        scale = max(1.0, float(np.max(np.abs(y))))
        assert float(np.max(np.abs(x - y))) / scale <= TRAJ_RTOL, f
    scale = max(1.0, float(np.max(np.abs(run.acc_i[0]))))
    assert float(np.max(np.abs(a - run.acc_i[0]))) / scale <= TRAJ_RTOL


def test_fast_cells_and_pairs_equal_exact(af3d, oracle):
    n = 900
    sys, fun, pp = _state("wall", n, 5)
    run = OracleRun(oracle, sys, fun, pp)
    got = {}
    for mode in (af3d.FP_EXACT, af3d.FP_FAST):
        with _engine(af3d, sys, fun, pp, run.cp, mode) as eng:
            eng.forces()
            cells, ids = eng.get_cells()
            pairs = set(map(tuple, eng.contact_pairs().tolist()))
            got[mode] = (cells, ids, pairs)
    e, f = got[af3d.FP_EXACT], got[af3d.FP_FAST]
    assert np.array_equal(e[0], f[0]) and np.array_equal(e[1], f[1]) and e[2] == f[2]


def test_fast_mode_switch_and_determinism(af3d, oracle):
    n = 1500
    sys, fun, pp = _state("dense", n, 8, time=0.0)
    run = OracleRun(oracle, sys, fun, pp)
    outs = []
    for _ in range(2):
        with _engine(af3d, sys, fun, pp, run.cp, af3d.FP_FAST) as eng:
            eng.forces()
            eng.swap_accel()
            eng.step(30)
            eng.set_fp_mode(af3d.FP_EXACT)      # switching drops the captured graphs
            eng.step(4)
            eng.set_fp_mode(af3d.FP_FAST)
            eng.step(30)
            outs.append(eng.export_particles()[0])
    assert outs[0].tobytes() == outs[1].tobytes()
    with af3d.Engine(sys, fun) as eng:
        with pytest.raises(af3d.EngineError):
            eng.set_fp_mode(7)


def test_fast_rotation_over_the_angle_range(af3d, oracle):
    """init_Verlet's rotation in fast mode -- Maclaurin series of sin(t)/t and (1 - cos t)/t^2
    below |dOmega| = 2^-5, rsqrt and sincos above -- against the oracle's sin/cos path, for
    rotation angles per step from 1e-9 to 0.2 rad on either side of the switch.  Rotation
    matrices and sphere centres within 1e-14 (absolute; entries are O(1)) per clump."""
    n = 600
    sys, fun, pp = _state("dense", n, 4, time=0.0)
    rng = np.random.default_rng(6)
    dt = float(sys["dt"])
    theta = np.concatenate([10.0 ** rng.uniform(-9, -0.7, n - 8),
                            2.0 ** -5 * np.array([0.999, 0.9999, 1.0, 1.0001, 1.001, 0.5, 2.0, 1e-3])])
    axis = rng.standard_normal((n, 3))
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    pp = pp.copy()
    pp["ww"] = axis * (theta / dt)[:, None]
    pp["vv"] = 0.0
    zero = np.zeros((n, 3))
    want = pp.copy()
    oracle.init_verlet(zero, zero, sys, want)
    with af3d.Engine(sys, fun, fp_mode=af3d.FP_FAST) as eng:
        eng.import_particles(pp)
        eng.init_verlet()
        got = eng.export_particles(with_accel=False)
    for f in ("Rmatx", "Rmaty", "Rmatz"):
        assert float(np.max(np.abs(got[f] - want[f]))) <= 1e-14, f
    assert float(np.max(np.abs(got["rr_s"] - want["rr_s"]))) <= 1e-14 * max(1.0, float(np.abs(want["rr_s"]).max()))


def test_integer_pipe_fp64_helpers(af3d):
    """The kernels convert and test doubles on the integer pipe (the FP64 pipe is the force
    kernel's bottleneck): conversions to float to nearest and toward +infinity, truncation to a
    64-bit integer, and the finiteness, non-zero and open-range tests must give the hardware's
    bits on every input: random bit patterns over the whole exponent range, rounding ties and
    their neighbours, float-range edges, zeros, subnormals, infinities and NaN."""
    import ctypes as C
    rng = np.random.default_rng(97)
    bits = rng.integers(0, 2 ** 63, 200000, dtype=np.int64).view(np.uint64)
    bits[::2] |= np.uint64(1 << 63)
    x = bits.view(np.float64)
    mags = (rng.random(200000) * 2 - 1) * 10.0 ** rng.integers(-45, 40, 200000)
    # ties of the float rounding: 29 low mantissa bits exactly half, and one unit either side
    base = (rng.random(20000) + 1.0) * 2.0 ** rng.integers(-120, 120, 20000)
    b = base.view(np.uint64) & ~np.uint64(0x1FFFFFFF)
    ties = np.concatenate([(b | np.uint64(0x10000000)), (b | np.uint64(0x0FFFFFFF)),
                           (b | np.uint64(0x10000001)), b]).view(np.float64)
    f32 = np.float32
    edges = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324, -5e-324, 2.2250738585072014e-308,
                      float(np.finfo(f32).max), -float(np.finfo(f32).max), float(np.finfo(f32).tiny),
                      float(np.finfo(f32).tiny) / 2, 3.4028235677973366e38, 3.4028235677973362e38,
                      1e39, 1.0, 1.0 - 2 ** -26, 1.0 + 2 ** -26, 1.0 - 2 ** -27, 1.0 + 2 ** -27,
                      9.765625e-04, np.nextafter(9.765625e-04, 0), 0.5, 2.0 ** 52, 2.0 ** 52 + 0.5,
                      2.0 ** 63, -2.0 ** 62, 123456789.99999, -0.999999])
    x = np.ascontiguousarray(np.concatenate([x, mags, ties, edges]))
    bad = np.zeros(len(x), dtype=np.int32)
    assert af3d.lib().af3d_check_fp64_bits(x.ctypes.data_as(C.c_void_p), len(x),
                                            bad.ctypes.data_as(C.c_void_p)) == 0
    assert not bad.any(), [(float(x[i]), int(bad[i])) for i in np.nonzero(bad)[0][:10]]
