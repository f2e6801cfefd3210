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


def _final(af3d, sys, fun, pp, steps=STEPS, phase=1, friction=0):
    """The exported final state of the forward run the adjoint differentiates."""
    with af3d.Engine(sys, fun, phase=phase, friction=friction) as eng:
        eng.import_particles(pp)
        eng.adjoint(steps, gradients=False)
        return eng.export_particles(with_accel=False)


def _J(af3d, sys, fun, pp, ref, steps=STEPS, phase=1, friction=0):
    """J - J(ref positions) from the exported final state (host, fixed order)."""
    p = _final(af3d, sys, fun, pp, steps, phase, friction)
    m = p["mass"]
    return float(np.sum(m * (_xrot(p, sys) - ref)) / np.sum(m))


def _runout_difference(pa, pb, sys, length):
    """J(pa) - J(pb) of the runout objective, l ln(sum m e^(x/l) / sum m), in a form free of
    cancellation: l log1p(sum m e^((xb - c)/l) expm1((xa - xb)/l) / sum m e^((xb - c)/l))."""
    xa, xb = _xrot(pa, sys), _xrot(pb, sys)
    m = pb["mass"]
    wb = m * np.exp((xb - float(np.max(xb))) / length)
    return length * float(np.log1p(np.sum(wb * np.expm1((xa - xb) / length)) / np.sum(wb)))


def _adjoint(af3d, sys, fun, pp, steps=STEPS, ckpt=40, phase=1, friction=0, runout=None):
    with af3d.Engine(sys, fun, phase=phase, friction=friction) as eng:
        eng.import_particles(pp)
        return eng.adjoint(steps, ckpt, runout=runout)


def _close(adj, fd, scale):
    return abs(adj - fd) <= TOL * max(abs(fd), 1e-3 * scale)


def _fd_agrees(Jat, h, adj, scale):
    """Whether the adjoint derivative `adj` agrees with finite differences of J(delta) = Jat(delta)
    at step h.  First the central difference, to the bar.  The forward run is only piecewise
    smooth: a perturbation can move a discrete event (a contact starting or ending a step
    earlier, a gate or the Coulomb branch switching) or change the rounding of a chaotic run,
    and the adjoint is the derivative of the piece the unperturbed run is on.  Where J is that
    rough at the scale h, its forward and backward differences disagree; the central
    difference is then uncertain by half their spread, and the adjoint must lie within it.
    (The tangent-linear tests check the same derivatives along the same pieces without finite
    differences.)  Returns (agrees, central difference, "central" or "rough")."""
    jp, jm = Jat(h), Jat(-h)
    central = (jp - jm) / (2 * h)
    if _close(adj, central, scale):
        return True, central, "central"
    j0 = Jat(0.0)
    spread = 0.5 * abs((jp - j0) / h - (j0 - jm) / h)
    return abs(adj - central) <= spread, central, "rough"


def test_adjoint_zero_steps(af3d, base):
    cfg, sys, fun, pp = base
    out = _adjoint(af3d, sys, fun, pp, steps=0)
    m = pp["mass"]
    want = np.stack([m * float(sys["cost"]), 0 * m, -m * float(sys["sint"])], 1) / m.sum()
    assert np.allclose(out["r0"], want, rtol=0, atol=1e-15)
    assert all(v == 0.0 for v in out["params"].values())
    assert np.all(out["R0"] == 0.0)


@pytest.mark.parametrize("friction", [0, 1])
@pytest.mark.parametrize("phase_time", [0.0, -0.5])
def test_adjoint_parameters_vs_finite_differences(af3d, base, phase_time, friction):
    """Both friction variants.  In the host variant (force_part.cu:224) a particle-particle
    contact whose tangential displacement survives the xi gate has |xi| <= mu N 1e-12, so its
    shear force is at most m mu N (1 + 2e-6 / dt), below mu N for the sphere masses and time
    step here: the Coulomb cap never fires, mu_pp enters only through the gate's decision, and
    dJ/dmu_pp is exactly zero.  The device variant (force_part.cu:487) also takes the Coulomb
    branch when the gate zeroed xi, so sliding contacts carry mu_pp and its gradient."""
    from oracle.pyoracle import PHASE_AVALANCHE, PHASE_FILL
    _, sys0, fun, pp = base
    sys = sys0.copy()
    sys["time"] = phase_time
    phase = PHASE_FILL if phase_time < 0 else PHASE_AVALANCHE
    ref = _xrot(pp, sys)
    out = _adjoint(af3d, sys, fun, pp, phase=phase, friction=friction)
    grads = out["params"]
    scale = max(abs(v * float(sys[k])) for k, v in grads.items())   # |dJ/dlog theta|
    rows, bad = [], []
    for k, g in grads.items():
        theta = float(sys[k])

        def Jat(delta, k=k, theta=theta):   # J at theta (1 + delta), in units of log theta
            sd = sys.copy()
            sd[k] = theta + delta * theta
            return _J(af3d, sd, fun, pp, ref, phase=phase, friction=friction)
        ok, fd, which = _fd_agrees(Jat, REL, g * theta, scale)
        rows.append((k, g * theta, fd, which))
        if not ok:
            bad.append(k)
    assert not bad, rows
    assert sum(abs(r[2]) > 1e-3 * scale for r in rows) >= 4, rows   # the run exercises both laws
    assert sum(r[3] != "central" for r in rows) <= 1, rows        # a rough parameter is the exception
    if friction == 0:
        assert grads["mu_pp"] == 0.0, rows
    else:
        assert abs(grads["mu_pp"] * float(sys["mu_pp"])) > 1e-3 * scale, rows


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


@pytest.mark.parametrize("friction", [0, 1])
@pytest.mark.parametrize("phase_time", [0.0, -0.5])
def test_adjoint_vs_tangent_linear_model(af3d, base, oracle, tangent, friction, phase_time):
    """The adjoint against the FP64 CPU tangent-linear model (the oracle over dual numbers) on
    the same run: eight directional derivatives -- each contact-law parameter, a random
    perturbation of positions and orientations, and one of velocities and spins -- to 1e-7, in
    both phases and both friction variants (the device variant differentiates the
    particle-particle Coulomb branch, force_part.cu:487)."""
    from oracle.pyoracle import CELL_PAR, PARTICLE, PHASE_AVALANCHE, PHASE_FILL, SYSTEM_PAR, state_tangent
    _, sys0, fun, pp = base
    sys = sys0.copy()
    sys["time"] = phase_time
    phase = PHASE_FILL if phase_time < 0 else PHASE_AVALANCHE
    out = _adjoint(af3d, sys, fun, pp, friction=friction, phase=phase)
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
    J, dJ, _ = tangent.run(sys, fun, cp, pp, STEPS, phase=phase, variant=friction, dsys=dsys, dpp=dpp)
    dR = np.stack([dpp[6]["Rmatx"], dpp[6]["Rmaty"], dpp[6]["Rmatz"]], 1)
    adj =[out["params"][k] * float(sys[k]) for k in names]
    adj.append(float(np.sum(out["r0"] * dr) + np.sum(out["R0"] * dR)))
    adj.append(float(np.sum(out["v0"] * dv) + np.sum(out["w0"] * dw)))
    adj = np.array(adj)
    assert out["J"] == pytest.approx(J, rel=1e-12)
    scale = float(np.abs(dJ).max())
    bad = [(k, adj[k], dJ[k]) for k in range(8) if abs(adj[k] - dJ[k]) > 1e-7 * max(abs(dJ[k]), 1e-3 * scale)]
    assert not bad, list(zip(adj, dJ))
    if friction == 1:
        assert abs(dJ[names.index("mu_pp")]) > 1e-3 * scale, list(zip(names, adj, dJ))


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


RUNOUT_L = 10.0   # cm: the soft maximum weights the clumps within a few l of the front


def test_runout_objective_value(af3d, base):
    """af3d_adjoint's runout J equals the host evaluation on the exported final state."""
    from avalancheflume3d_gb300.adjoint import runout
    _, sys, fun, pp = base
    with af3d.Engine(sys, fun) as eng:
        eng.import_particles(pp)
        J = eng.adjoint(STEPS, gradients=False, runout=RUNOUT_L)["J"]
        p = eng.export_particles(with_accel=False)
    assert J == pytest.approx(runout(p, sys, RUNOUT_L), rel=1e-13)
    assert J > np.percentile(_xrot(p, sys), 95)


@pytest.mark.parametrize("friction", [0, 1])
def test_runout_gradients_vs_finite_differences(af3d, base, friction):
    """Gradients of the runout objective (a soft maximum of the downslope positions, length
    scale 10 cm) with respect to the contact-law parameters and to the initial positions of the
    clumps nearest the front, against central finite differences of the same forward run."""
    from oracle.pyoracle import sphere_centres
    _, sys, fun, pp = base
    out = _adjoint(af3d, sys, fun, pp, friction=friction, runout=RUNOUT_L)
    grads = out["params"]
    base_state = _final(af3d, sys, fun, pp, friction=friction)
    scale = max(abs(v * float(sys[k])) for k, v in grads.items())
    rows, bad = [], []
    for k, g in grads.items():
        h = REL * float(sys[k])
        sp, sm = sys.copy(), sys.copy()
        sp[k] += h
        sm[k] -= h
        fd = (_runout_difference(_final(af3d, sp, fun, pp, friction=friction), base_state, sys, RUNOUT_L) -
              _runout_difference(_final(af3d, sm, fun, pp, friction=friction), base_state, sys, RUNOUT_L)) / (2 * h)
        rows.append((k, g * float(sys[k]), fd * float(sys[k])))
        if not _close(g * float(sys[k]), fd * float(sys[k]), scale):
            bad.append(k)
    assert not bad, rows
    assert sum(abs(r[2]) > 1e-3 * scale for r in rows) >= 2, rows
    g = out["r0"]
    pick = np.argsort(-_xrot(pp, sys))[:3]
    h = 1e-6 * float(pp["radius"][0])
    gscale = float(np.abs(g).max())
    for i in pick:
        for ax in (0, 2):
            qp, qm = pp.copy(), pp.copy()
            qp["rr"][i, ax] += h
            qm["rr"][i, ax] -= h
            sphere_centres(qp)
            sphere_centres(qm)
            fd = (_runout_difference(_final(af3d, sys, fun, qp, friction=friction), base_state, sys, RUNOUT_L) -
                  _runout_difference(_final(af3d, sys, fun, qm, friction=friction), base_state, sys, RUNOUT_L)) / (2 * h)
            rows.append((int(i), ax, g[i, ax], fd))
            if not _close(g[i, ax], fd, gscale):
                bad.append((int(i), ax))
    assert not bad, rows


def _moved(pp, r0):
    """pp with its clump centres at r0 (the sphere centres follow)."""
    from oracle.pyoracle import sphere_centres
    q = pp.copy()
    q["rr"] = r0
    sphere_centres(q)
    return q


def test_flume_run_function_autograd(af3d, base):
    """The torch.autograd.Function: torch.autograd.grad of J with respect to the initial
    positions equals the engine's adjoint, for one flume and (scaled per flume by the incoming
    gradient) for an ensemble."""
    torch = pytest.importorskip("torch")
    from avalancheflume3d_gb300.adjoint import flume_run_function
    _, sys, fun, pp = base
    FlumeRun = flume_run_function()
    steps, ckpt = 40, 20

    def make(r0):
        eng = af3d.Engine(sys, fun)
        eng.import_particles(_moved(pp, r0))
        return eng

    r0 = torch.tensor(pp["rr"], dtype=torch.float64, requires_grad=True)
    J = FlumeRun.apply(r0, make, steps, ckpt, None)
    (g,) = torch.autograd.grad(3.0 * J, r0)
    want = _adjoint(af3d, sys, fun, pp, steps=steps, ckpt=ckpt)
    assert float(J.detach()) == pytest.approx(want["J"], rel=1e-13)
    assert np.allclose(g.numpy(), 3.0 * want["r0"], rtol=1e-9, atol=1e-12 * float(np.abs(want["r0"]).max()))
    # an ensemble of two copies with different friction: J has one entry per flume
    sys2 = sys.copy()
    sys2["mu_pw"] = 0.25
    sys2["fr_fact_pw"] = 0.25 / 1.0e12
    syss, funs = np.stack([sys, sys2]), np.stack([fun, fun])

    def make_ens(r0):
        eng = af3d.Engine(syss, funs)
        eng.import_particles(np.concatenate([_moved(pp, r0[:N]), _moved(pp, r0[N:])]))
        return eng

    r0e = torch.tensor(np.concatenate([pp["rr"], pp["rr"]]), dtype=torch.float64, requires_grad=True)
    Je = FlumeRun.apply(r0e, make_ens, steps, ckpt, None)
    assert Je.shape == (2,)
    (ge,) = torch.autograd.grad(2.0 * Je[0] - 5.0 * Je[1], r0e)
    with af3d.Engine(syss, funs) as eng:
        eng.import_particles(np.concatenate([pp, pp]))
        we = eng.adjoint(steps, ckpt)
    assert np.allclose(Je.detach().numpy(), we["J"], rtol=1e-13)
    wg = np.concatenate([2.0 * we["r0"][:N], -5.0 * we["r0"][N:]])
    assert np.allclose(ge.numpy(), wg, rtol=1e-9, atol=1e-12 * float(np.abs(wg).max()))


def test_adjoint_configs4_flume_vs_tangent_linear_model(af3d, oracle, tangent):
    """The adjoint configuration itself: 32,768 clumps of the 80 cm x 4 cm flume at 35 deg (dense
    bed layer), the device friction variant (every parameter has a gradient), 1,000 exact steps
    with a checkpoint every 250 (three segments recomputed), against the FP64 tangent-linear model
    on the same run (all host threads): the six contact-law parameters and one random
    perturbation of the positions and orientations, to 1e-7.  (Over this many clumps and steps,
    finite differences of J are dominated by discrete events -- contacts starting a step
    earlier or later under the perturbation -- which the piecewise-smooth derivative excludes by
    definition; the tangent-linear model follows the same pieces.)"""
    import os
    from oracle.pyoracle import CELL_PAR, PARTICLE, SYSTEM_PAR, state_tangent
    from avalancheflume3d_gb300.workloads import flume_2k, flume_state
    cfg = flume_2k(n=32768, tilt_deg=35.0, Lflume=80.0, layout="bed")
    sys, fun, pp = flume_state(cfg)
    n, steps = len(pp), 1000
    out = _adjoint(af3d, sys, fun, pp, steps=steps, ckpt=250, friction=1)
    names = list(out["params"])
    dsys = np.zeros(7, dtype=SYSTEM_PAR)
    for k, name in enumerate(names):
        dsys[k][name] = float(sys[name])
    rng = np.random.default_rng(41)
    dr, dphi = rng.standard_normal((n, 3)) * float(sys["rmax"]), rng.standard_normal((n, 3))
    dpp = np.zeros((7, n), dtype=PARTICLE)
    dpp[6] = state_tangent(pp, sys, dr=dr, dphi=dphi)
    cp = np.zeros((), dtype=CELL_PAR)
    cp["ntags"] = 9
    cp["rr_max"], cp["rr_min"] = oracle.cell_dim(pp, sys)
    oracle.grid_from_bbox(cp, sys)
    tangent.set_threads(os.cpu_count() or 1)
    J, dJ, _ = tangent.run(sys, fun, cp, pp, steps, variant=1, dsys=dsys, dpp=dpp)
    dR = np.stack([dpp[6]["Rmatx"], dpp[6]["Rmaty"], dpp[6]["Rmatz"]], 1)
    adj = [out["params"][k] * float(sys[k]) for k in names]
    adj.append(float(np.sum(out["r0"] * dr) + np.sum(out["R0"] * dR)))
    assert out["J"] == pytest.approx(J, rel=1e-12)
    scale = float(np.abs(dJ).max())
    bad = [(k, adj[k], dJ[k]) for k in range(7) if abs(adj[k] - dJ[k]) > 1e-7 * max(abs(dJ[k]), 1e-3 * scale)]
    assert not bad, list(zip(names + ["state"], adj, dJ))
    pscale = float(np.abs(dJ[:6]).max())
    assert all(abs(d) > 1e-4 * pscale for d in dJ[:6]), list(zip(names, dJ))
