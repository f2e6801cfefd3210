"""Batched ensemble: several independent flumes in one context (af3d_create_ensemble).

Each flume of an ensemble must evolve exactly as it does alone: forces bit-exact against the
oracle run on that flume alone, trajectories bit-identical to a single-flume context and within
the trajectory tolerance of the oracle, per-flume grids derived on the device bit-exact, and no
contact pair between clumps of different flumes.
"""
import numpy as np
import pytest

from oracle.pyoracle import FRICTION_DEV, FRICTION_HST, PARTICLE, PHASE_AVALANCHE, OracleRun, dense_state
from tests.states import flume_system, wall_state

pytestmark = pytest.mark.gpu

TRAJ_RTOL = 1e-8

# (clumps, tilt, mu_pp, mu_pw, restitution, state, seed): material, geometry and sizes differ
FLUMES = [
    (300, 35.0, 0.5, 0.4, 0.5, "wall", 31),
    (520, 30.0, 0.3, 0.6, 0.7, "dense", 32),
    (12, 40.0, 0.5, 0.4, 0.5, "wall", 33),
    (0, 35.0, 0.5, 0.4, 0.5, "wall", 35),
    (260, 42.0, 0.8, 0.2, 0.3, "dense", 34),
]
ONE = (1, 38.0, 0.6, 0.5, 0.4, "wall", 36)   # cell_dim gives a degenerate grid around one clump


@pytest.fixture(scope="module")
def af3d():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    af3d.lib()
    return af3d


def _flumes(time=0.0, specs=FLUMES):
    out = []
    for n, tilt, mu_pp, mu_pw, eps, kind, seed in specs:
        sys, fun = flume_system(n, tilt=tilt, mu_pp=mu_pp, mu_pw=mu_pw, eps=eps, time=time)
        if n == 0:
            pp = np.zeros(0, dtype=PARTICLE)
        elif kind == "wall":
            pp = wall_state(n, seed, sys)
        else:
            pp = dense_state(n, seed, sys, box=(1.0, 8.0, 26.0))
        out.append((sys, fun, pp))
    return out


def _grid(oracle, sys, fun, pp):
    """The oracle's cell_dim grid, with a fixed box where one clump (or none) gives a degenerate
    one."""
    from oracle.pyoracle import CELL_PAR, grid_from_bbox
    if len(pp) == 0:
        cp = np.zeros((), dtype=CELL_PAR)
        cp["ntags"] = 9
        cp["rr_min"], cp["rr_max"] = (0.0, 0.0, 0.0), (5.0, 5.0, 5.0)
        grid_from_bbox(cp, sys)
        return cp
    run = OracleRun(oracle, sys, fun, pp)
    if int(run.cp["ncell3"]) > 0:
        return run.cp
    cp = np.zeros((), dtype=CELL_PAR)
    cp["ntags"] = 9
    cp["rr_min"], cp["rr_max"] = pp["rr"].min(0) - 1.0, pp["rr"].max(0) + 1.0
    grid_from_bbox(cp, sys)
    return cp


def _ensemble(af3d, flumes, grids=None, acc=None, anga=None, friction=FRICTION_HST):
    sys = np.stack([f[0] for f in flumes])
    fun = np.stack([f[1] for f in flumes])
    eng = af3d.Engine(sys, fun, friction=friction)
    if grids is not None:
        for f, g in enumerate(grids):
            eng.set_flume_grid(f, g)
    eng.import_particles(np.concatenate([f[2] for f in flumes]), acc, anga)
    return eng


def _same(a, b):
    return np.asarray(a).tobytes() == np.asarray(b).tobytes()


@pytest.mark.parametrize("friction", [FRICTION_HST, FRICTION_DEV])
def test_ensemble_forces_bit_exact_per_flume(af3d, oracle, friction):
    flumes = _flumes(time=0.001, specs=FLUMES + [ONE])
    grids = [_grid(oracle, *f) for f in flumes]
    runs = [OracleRun(oracle, s, u, p, cp=g) if len(p) else None for (s, u, p), g in zip(flumes, grids)]
    for r in runs:
        assert r is None or r.forces(PHASE_AVALANCHE, friction) == 0
    with _ensemble(af3d, flumes, grids, friction=friction) as eng:
        assert eng.flume_count() == len(flumes)
        eng.forces()
        F, T = eng.get_forces()
        a, al = eng.get_accels()
        for f, r in enumerate(runs):
            if r is None:
                continue
            sl = eng.flume_slice(f)
            assert _same(F[sl], r.bufs["F"]) and _same(T[sl], r.bufs["T"]), "flume %d forces" % f
            assert _same(a[sl], r.acc_f[0]) and _same(al[sl], r.acc_f[1]), "flume %d accels" % f


def test_ensemble_contact_pairs_stay_inside_flumes(af3d, oracle):
    flumes = _flumes(time=0.001)
    grids = [_grid(oracle, *f) for f in flumes]
    with _ensemble(af3d, flumes, grids) as eng:
        eng.forces()
        pairs = eng.contact_pairs()
        first = eng.first_id
    fl = np.searchsorted(first, pairs[:, :2], side="right") - 1
    assert len(pairs) > 0 and np.array_equal(fl[:, 0], fl[:, 1])
    for f, (s, u, p) in enumerate(flumes):
        if len(p) == 0:
            continue
        with af3d.Engine(s, u) as one:
            one.set_grid(grids[f])
            one.import_particles(p)
            one.forces()
            want = set(map(tuple, (one.contact_pairs() + [first[f], first[f], 0]).tolist()))
        got = set(map(tuple, pairs[fl[:, 0] == f].tolist()))
        assert got == want, "flume %d" % f


def test_ensemble_device_regrid_per_flume(af3d, oracle):
    flumes = _flumes()
    with _ensemble(af3d, flumes) as eng:      # first import derives every flume's grid
        grids = [eng.get_flume_grid(f) for f in range(len(flumes))]
    for (s, u, p), g in zip(flumes, grids):
        if len(p):
            assert _same(g, OracleRun(oracle, s, u, p).cp)
        else:                                 # a flume without clumps gets a one-cell grid
            assert int(g["ncell3"]) == 1


def test_ensemble_trajectory_matches_single_flumes(af3d, oracle):
    """100 fused steps (one device re-grid after the first): every flume bit-identical to a
    single-flume context and within the trajectory tolerance of the oracle."""
    flumes = _flumes(time=0.0)
    grids = [_grid(oracle, *f) for f in flumes]
    runs = [OracleRun(oracle, s, u, p, cp=g) if len(p) else None for (s, u, p), g in zip(flumes, grids)]
    for r in runs:
        assert r is None or r.seed_accel() == 0
    acc = np.concatenate([r.acc_i[0] if r else np.zeros((0, 3)) for r in runs])
    anga = np.concatenate([r.acc_i[1] if r else np.zeros((0, 3)) for r in runs])
    with _ensemble(af3d, flumes, grids, acc.copy(), anga.copy()) as eng:
        eng.step(100)
        p, a, _ = eng.export_particles()
        t = float(eng.get_flume_system(2)["time"])
        g_after = [eng.get_flume_grid(f) for f in range(len(flumes))]
        slices = [eng.flume_slice(f) for f in range(len(flumes))]
    for f, ((s, u, p0), g, r) in enumerate(zip(flumes, grids, runs)):
        if r is None:
            assert _same(g_after[f], g)       # a flume without clumps keeps its grid
            continue
        sl = slices[f]
        with af3d.Engine(s, u) as one:
            one.set_grid(g)
            one.import_particles(p0, acc[sl].copy(), anga[sl].copy())
            one.step(100)
            q, b, _ = one.export_particles()
            assert _same(one.get_grid(), g_after[f])
        assert _same(p[sl], q) and _same(a[sl], b), "flume %d differs from its single-flume run" % f
        assert r.step(100, cc0=0) == 0
        for fld in ("rr", "vv", "ww", "Rmatx", "rr_s"):
            scale = max(1.0, float(np.max(np.abs(r.pp[fld]))))
            err = float(np.max(np.abs(p[sl][fld] - r.pp[fld]))) / scale
            assert err <= TRAJ_RTOL, "flume %d %s: %.3e" % (f, fld, err)
    assert t == float(runs[0].sys["time"])
    assert len({int(g["ncell3"]) for g in g_after}) > 1      # the flumes were re-gridded apart


def test_ensemble_rejects_mixed_dt(af3d):
    flumes = _flumes(specs=FLUMES[:2])
    sys = np.stack([f[0] for f in flumes])
    fun = np.stack([f[1] for f in flumes])
    sys[1]["dt"] = 2 * sys[0]["dt"]
    sys[1]["hdt"] = sys[0]["dt"]
    with pytest.raises(af3d.EngineError) as e:
        af3d.Engine(sys, fun)
    assert e.value.code == 1
    with af3d.Engine(np.stack([flumes[0][0]] * 2), np.stack([flumes[0][1]] * 2)) as eng:
        with pytest.raises(af3d.EngineError):
            eng.get_flume_grid(2)
