"""The hand-written adjoint of the exact step (af3d_adjoint) against central finite differences
of the same forward run (relative step 1e-6) over a short horizon: gradients of J, the
mass-weighted mean downslope position after the start-up force pass and K steps, with respect to
the contact-law parameters of system_par, to the configuration's (mu_pp, mu_wall, restitution,
kn), and to initial positions and orientations.  The bar is 1e-4 relative.

The finite differences read J from the exported final state on the host, as a displacement from
a fixed reference, in a fixed summation order, so they are free of the device reduction's
rounding; forward runs in exact mode are deterministic."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 100
REL = 1e-6
TOL = 1e-4
N = 600


@pytest.fixture(scope="module")
def af3d():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    af3d.lib()
    return af3d


def _material_system(mu_pp=0.5, mu_pw=0.4, restitution=0.5, kn=1.0e7, time=0.0):
    """system_par of the 600-clump test flume from the configuration's material parameters."""
    from avalancheflume3d_gb300.workloads import FlumeConfig
    from tests.states import flume_system
    t_coll = FlumeConfig(n=N, kn=kn, restitution=restitution).t_coll
    return flume_system(N, mu_pp=mu_pp, mu_pw=mu_pw, eps=restitution, t_coll=t_coll, time=time)


@pytest.fixture(scope="module")
def base():
    """Six clusters touching every boundary type (hopper, funnel, corners, side walls, bed) and a
    dense block, with random velocities and spins: every routine's reverse is exercised."""
    from tests.states import wall_state
    sys, fun = _material_system()
    pp = wall_state(N, 77, sys)
    return None, sys, fun, pp


def _xrot(pp, sys):
    return pp["rr"][:, 0] * float(sys["cost"]) - pp["rr"][:, 2] * float(sys["sint"])


def _J(af3d, sys, fun, pp, ref, steps=STEPS, phase=1):
    """J - J(ref positions) from the exported final state (host, fixed order)."""
    with af3d.Engine(sys, fun, phase=phase) as eng:
        eng.import_particles(pp)
        eng.adjoint(steps, gradients=False)
        p = eng.export_particles(with_accel=False)
    m = p["mass"]
    return float(np.sum(m * (_xrot(p, sys) - ref)) / np.sum(m))


def _adjoint(af3d, sys, fun, pp, steps=STEPS, ckpt=40, phase=1):
    with af3d.Engine(sys, fun, phase=phase) as eng:
        eng.import_particles(pp)
        return eng.adjoint(steps, ckpt)


def _close(adj, fd, scale):
    return abs(adj - fd) <= TOL * max(abs(fd), 1e-3 * scale)


def test_adjoint_zero_steps(af3d, base):
    cfg, sys, fun, pp = base
    out = _adjoint(af3d, sys, fun, pp, steps=0)
    m = pp["mass"]
    want = np.stack([m * float(sys["cost"]), 0 * m, -m * float(sys["sint"])], 1) / m.sum()
    assert np.allclose(out["r0"], want, rtol=0, atol=1e-15)
    assert all(v == 0.0 for v in out["params"].values())
    assert np.all(out["R0"] == 0.0)


@pytest.mark.parametrize("phase_time", [0.0, -0.5])
def test_adjoint_parameters_vs_finite_differences(af3d, base, phase_time):
    from oracle.pyoracle import PHASE_AVALANCHE, PHASE_FILL
    _, sys0, fun, pp = base
    sys = sys0.copy()
    sys["time"] = phase_time
    phase = PHASE_FILL if phase_time < 0 else PHASE_AVALANCHE
    ref = _xrot(pp, sys)
    out = _adjoint(af3d, sys, fun, pp, phase=phase)
    grads = out["params"]
    scale = max(abs(v * float(sys[k])) for k, v in grads.items())   # |dJ/dlog theta|
    rows, bad = [], []
    for k, g in grads.items():
        h = REL * float(sys[k])
        sp, sm = sys.copy(), sys.copy()
        sp[k] += h
        sm[k] -= h
        fd = (_J(af3d, sp, fun, pp, ref, phase=phase) - _J(af3d, sm, fun, pp, ref, phase=phase)) / (2 * h)
        rows.append((k, g * float(sys[k]), fd * float(sys[k])))
        if not _close(g * float(sys[k]), fd * float(sys[k]), scale):
            bad.append(k)
    assert not bad, rows
    assert sum(abs(r[2]) > 1e-3 * scale for r in rows) >= 4, rows   # the run exercises both laws


def test_adjoint_positions_vs_finite_differences(af3d, base):
    from oracle.pyoracle import sphere_centres
    cfg, sys, fun, pp = base
    ref = _xrot(pp, sys)
    out = _adjoint(af3d, sys, fun, pp)
    g = out["r0"]
    # clumps with the largest gradients beyond the direct term: those in contact
    direct = np.stack([pp["mass"] * float(sys["cost"]), 0 * pp["mass"], -pp["mass"] * float(sys["sint"])], 1)
    direct /= pp["mass"].sum()
    pick = np.argsort(-np.abs(g - direct).sum(1))[:4]
    h = 1e-6 * float(pp["radius"][0])
    scale = float(np.abs(g).max())
    rows, bad = [], []
    for i in pick:
        for ax in range(3):
            qp, qm = pp.copy(), pp.copy()
            qp["rr"][i, ax] += h
            qm["rr"][i, ax] -= h
            sphere_centres(qp)
            sphere_centres(qm)
            fd = (_J(af3d, sys, fun, qp, ref) - _J(af3d, sys, fun, qm, ref)) / (2 * h)
            rows.append((int(i), ax, g[i, ax], fd))
            if not _close(g[i, ax], fd, scale):
                bad.append((int(i), ax))
    assert not bad, rows


def test_adjoint_orientations_vs_finite_differences(af3d, base):
    from avalancheflume3d_gb300.adjoint import rotation_gradient
    from oracle.pyoracle import sphere_centres
    cfg, sys, fun, pp = base
    ref = _xrot(pp, sys)
    out = _adjoint(af3d, sys, fun, pp)
    R = np.stack([pp["Rmatx"], pp["Rmaty"], pp["Rmatz"]], 1)
    gphi = rotation_gradient(R, out["R0"])
    pick = np.argsort(-np.abs(gphi).sum(1))[:3]
    h = 1e-6
    scale = float(np.abs(gphi).max())
    rows, bad = [], []
    for i in pick:
        for ax in range(3):
            fds = []
            for sgn in (1.0, -1.0):
                q = pp.copy()
                k = np.zeros(3)
                k[ax] = sgn * h
                K = np.array([[0, -k[2], k[1]], [k[2], 0, -k[0]], [-k[1], k[0], 0]])
                Rot = np.eye(3) + np.sin(h) / h * K + (1 - np.cos(h)) / h ** 2 * K @ K
                Rn = Rot @ R[i]
                q["Rmatx"][i], q["Rmaty"][i], q["Rmatz"][i] = Rn[0], Rn[1], Rn[2]
                sphere_centres(q)
                fds.append(_J(af3d, sys, fun, q, ref))
            fd = (fds[0] - fds[1]) / (2 * h)
            rows.append((int(i), ax, gphi[i, ax], fd))
            if not _close(gphi[i, ax], fd, scale):
                bad.append((int(i), ax))
    assert not bad, rows


def test_adjoint_vs_tangent_linear_model(af3d, base, oracle, tangent):
    """The adjoint against the FP64 CPU tangent-linear model (the oracle over dual numbers) on
    the same run: eight directional derivatives -- each contact-law parameter, a random
    perturbation of positions and orientations, and one of velocities and spins -- to 1e-7."""
    from oracle.pyoracle import CELL_PAR, PARTICLE, SYSTEM_PAR, state_tangent
    _, sys, fun, pp = base
    out = _adjoint(af3d, sys, fun, pp)
    rng = np.random.default_rng(17)
    names = list(out["params"])
    dsys = np.zeros(tangent.ndirs, dtype=SYSTEM_PAR)
    for k, name in enumerate(names):
        dsys[k][name] = float(sys[name])
    dr, dphi = rng.standard_normal((N, 3)) * float(sys["rmax"]), rng.standard_normal((N, 3))
    dv, dw = rng.standard_normal((N, 3)) * 10.0, rng.standard_normal((N, 3)) * 30.0
    dpp = np.zeros((tangent.ndirs, N), dtype=PARTICLE)
    dpp[6] = state_tangent(pp, sys, dr=dr, dphi=dphi)
    dpp[7] = state_tangent(pp, sys, dv=dv, dw=dw)
    # a coarse grid: the contacts found do not depend on the cell side
    cp = np.zeros((), dtype=CELL_PAR)
    cp["ntags"] = 128
    cp["rr_max"], cp["rr_min"] = oracle.cell_dim(pp, sys)
    s8 = sys.copy()
    s8["rmax"] *= 8.0
    oracle.grid_from_bbox(cp, s8)
    J, dJ, _ = tangent.run(sys, fun, cp, pp, STEPS, dsys=dsys, dpp=dpp)
    dR = np.stack([dpp[6]["Rmatx"], dpp[6]["Rmaty"], dpp[6]["Rmatz"]], 1)
    adj =[out["params"][k] * float(sys[k]) for k in names]
    adj.append(float(np.sum(out["r0"] * dr) + np.sum(out["R0"] * dR)))
    adj.append(float(np.sum(out["v0"] * dv) + np.sum(out["w0"] * dw)))
    adj = np.array(adj)
    assert out["J"] == pytest.approx(J, rel=1e-12)
    scale = float(np.abs(dJ).max())
    bad = [(k, adj[k], dJ[k]) for k in range(8) if abs(adj[k] - dJ[k]) > 1e-7 * max(abs(dJ[k]), 1e-3 * scale)]
    assert not bad, list(zip(adj, dJ))


def test_adjoint_configuration_chain_vs_finite_differences(af3d, base):
    from avalancheflume3d_gb300.adjoint import config_gradients
    from avalancheflume3d_gb300.workloads import FlumeConfig
    _, sys, fun, pp = base
    ref = _xrot(pp, sys)
    vals = {"mu_pp": 0.5, "mu_pw": 0.4, "restitution": 0.5, "kn": 1.0e7}
    cfg = FlumeConfig(n=N, **{"mu_pp": 0.5, "mu_pw": 0.4, "restitution": 0.5, "kn": 1.0e7})
    g = config_gradients(cfg, _adjoint(af3d, sys, fun, pp)["params"])
    scale = max(abs(g[k] * v) for k, v in vals.items())
    rows, bad = [], []
    for k, v in vals.items():
        h = REL * v
        Js = []
        for sgn in (1.0, -1.0):
            s2, f2 = _material_system(**{**vals, k: v + sgn * h})
            Js.append(_J(af3d, s2, f2, pp, ref))
        fd = (Js[0] - Js[1]) / (2 * h)
        rows.append((k, g[k] * v, fd * v))
        if not _close(g[k] * v, fd * v, scale):
            bad.append(k)
    assert not bad, rows


def test_adjoint_checkpoint_interval_does_not_matter(af3d, base):
    cfg, sys, fun, pp = base
    a = _adjoint(af3d, sys, fun, pp, steps=120, ckpt=120)
    b = _adjoint(af3d, sys, fun, pp, steps=120, ckpt=7)
    assert a["J"] == pytest.approx(b["J"], rel=1e-14)   # a device reduction: order varies
    # gradients are sums formed with FP64 atomics, whose order varies from run to run
    for k in a["params"]:
        assert a["params"][k] == pytest.approx(b["params"][k], rel=1e-9, abs=1e-12 * max(abs(a["params"][k]), 1e-300))
    assert np.allclose(a["r0"], b["r0"], rtol=1e-9, atol=1e-12 * float(np.abs(a["r0"]).max()))


def test_ensemble_adjoint_equals_each_flume_alone(af3d):
    """One backward sweep over an ensemble gives every flume's own J and gradients: those of the
    flume run alone (up to the order of the FP64 atomic sums)."""
    from tests.states import flume_system, wall_state
    specs = [(300, 35.0, 0.5, 0.4, 0.5, 41), (180, 30.0, 0.3, 0.6, 0.7, 42), (240, 40.0, 0.8, 0.2, 0.3, 43)]
    flumes = []
    for n, tilt, mu_pp, mu_pw, eps, seed in specs:
        sys, fun = flume_system(n, tilt=tilt, mu_pp=mu_pp, mu_pw=mu_pw, eps=eps)
        flumes.append((sys, fun, wall_state(n, seed, sys)))
    steps, ckpt = 60, 25
    with af3d.Engine(np.stack([f[0] for f in flumes]), np.stack([f[1] for f in flumes])) as eng:
        eng.import_particles(np.concatenate([f[2] for f in flumes]))
        ens = eng.adjoint(steps, ckpt)
    assert ens["J"].shape == (3,)
    lo = 0
    for f, (sys, fun, pp) in enumerate(flumes):
        one = _adjoint(af3d, sys, fun, pp, steps=steps, ckpt=ckpt)
        hi = lo + len(pp)
        assert ens["J"][f] == pytest.approx(one["J"], rel=1e-13)
        for k, v in one["params"].items():
            assert ens["params"][k][f] == pytest.approx(v, rel=1e-9, abs=1e-12 * max(abs(v), 1e-300)), (f, k)
        assert any(abs(v) > 0 for v in one["params"].values())
        for key in ("r0", "v0", "w0", "R0"):
            a, b = ens[key][lo:hi], one[key]
            assert np.allclose(a, b, rtol=1e-9, atol=1e-12 * float(np.abs(b).max())), (f, key)
        lo = hi


def test_adjoint_with_overflowed_contact_lists(af3d, base, oracle, tangent):
    """Five clumps piled almost on one spot give a clump more sphere contacts than its item lists
    hold (32), every step: its contacts run by the per-clump walk in the forward pass, and the
    reverse rebuilds that step's cell structure for it.  Checked against the tangent-linear model
    like the regular run (to 1e-7), with the overflow itself checked on the initial state."""
    from oracle.pyoracle import CELL_PAR, PARTICLE, SYSTEM_PAR, rotate_slope, sphere_centres, state_tangent
    _, sys, fun, pp0 = base
    pp = pp0.copy()
    rmax = float(sys["rmax"])
    i0 = N - 40   # inside the dense block on the bed
    rng = np.random.default_rng(23)
    pile = np.arange(i0 + 1, i0 + 5)
    pp["rr"][pile] = pp["rr"][i0] + (rng.random((len(pile), 3)) - 0.5) * 0.6 * rmax
    sphere_centres(pp)
    rotate_slope(pp, sys)
    s = pp["rr_s"]
    d = np.linalg.norm(s[i0][:, None, None, :] - s[np.arange(N) != i0][None, :, :, :], axis=-1)
    assert int(np.sum(d < 2.0 * pp["radius"][i0])) > 40
    steps = 40
    out = _adjoint(af3d, sys, fun, pp, steps=steps, ckpt=15)
    rng = np.random.default_rng(29)
    names = list(out["params"])
    dsys = np.zeros(tangent.ndirs, dtype=SYSTEM_PAR)
    for k, name in enumerate(names):
        dsys[k][name] = float(sys[name])
    dr, dphi = rng.standard_normal((N, 3)) * rmax, rng.standard_normal((N, 3))
    dv, dw = rng.standard_normal((N, 3)) * 10.0, rng.standard_normal((N, 3)) * 30.0
    dpp = np.zeros((tangent.ndirs, N), dtype=PARTICLE)
    dpp[6] = state_tangent(pp, sys, dr=dr, dphi=dphi)
    dpp[7] = state_tangent(pp, sys, dv=dv, dw=dw)
    cp = np.zeros((), dtype=CELL_PAR)
    cp["ntags"] = 128
    cp["rr_max"], cp["rr_min"] = oracle.cell_dim(pp, sys)
    s8 = sys.copy()
    s8["rmax"] *= 8.0
    oracle.grid_from_bbox(cp, s8)
    J, dJ, _ = tangent.run(sys, fun, cp, pp, steps, dsys=dsys, dpp=dpp)
    dR = np.stack([dpp[6]["Rmatx"], dpp[6]["Rmaty"], dpp[6]["Rmatz"]], 1)
    adj = [out["params"][k] * float(sys[k]) for k in names]
    adj.append(float(np.sum(out["r0"] * dr) + np.sum(out["R0"] * dR)))
    adj.append(float(np.sum(out["v0"] * dv) + np.sum(out["w0"] * dw)))
    adj = np.array(adj)
    assert out["J"] == pytest.approx(J, rel=1e-12)
    scale = float(np.abs(dJ).max())
    bad = [(k, adj[k], dJ[k]) for k in range(8) if abs(adj[k] - dJ[k]) > 1e-7 * max(abs(dJ[k]), 1e-3 * scale)]
    assert not bad, list(zip(adj, dJ))
