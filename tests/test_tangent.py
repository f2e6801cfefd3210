"""The FP64 tangent-linear model (oracle/af3d_tangent.cpp), pinned before it serves as the
forward-mode reference of the adjoint:

  * its value path is the oracle's: the final state after the start-up force pass and K steps
    is bit-identical to the oracle run's (same operations, same order, no contraction)
  * its directional derivatives -- along each contact-law parameter of system_par and along
    random perturbations of the initial positions, orientations, velocities and spins -- agree
    with central finite differences (relative step 1e-6) of the oracle itself to 1e-4 (the
    differences' own truncation error is ~1e-5 here)

The runs use a coarse cell grid (cells 8x the usual side, 128 slots each): the contacts found
do not depend on the cell side, and the sparse test state would otherwise spend its time
clearing a grid of ten million cells every step.
"""
import numpy as np
import pytest

from oracle.pyoracle import (CELL_PAR, PARTICLE, PHASE_AVALANCHE, PHASE_FILL, SYSTEM_PAR, OracleRun,
                             state_tangent)
from tests.states import flume_system, wall_state

N = 200
STEPS = 40
PARAMS = ("kappa_pp", "gamma_pp", "mu_pp", "kappa_pw", "gamma_pw", "mu_pw")
FIELDS = [f for f in PARTICLE.names]


def _case(time=0.0):
    sys, fun = flume_system(N, time=time)
    pp = wall_state(N, 91, sys)
    return sys, fun, pp


def _coarse_grid(oracle, sys, pp):
    cp = np.zeros((), dtype=CELL_PAR)
    cp["ntags"] = 128
    cp["rr_max"], cp["rr_min"] = oracle.cell_dim(pp, sys)
    s8 = sys.copy()
    s8["rmax"] *= 8.0
    oracle.grid_from_bbox(cp, s8)
    return cp


def _xrot(pp, sys):
    return pp["rr"][:, 0] * float(sys["cost"]) - pp["rr"][:, 2] * float(sys["sint"])


def _J(run_pp, sys, ref):
    m = run_pp["mass"]
    return float(np.sum(m * (_xrot(run_pp, sys) - ref)) / np.sum(m))


def _oracle_final(oracle, sys, fun, cp, pp, phase):
    run = OracleRun(oracle, sys, fun, pp, cp=cp)
    assert run.seed_accel(phase) == 0
    assert run.step(STEPS, phase) == 0
    return run.pp


def _shift(pp, t, h):
    q = pp.copy()
    for f in FIELDS:
        q[f] = pp[f] + h * t[f]
    return q


@pytest.mark.parametrize("phase", [PHASE_AVALANCHE, PHASE_FILL])
def test_tangent_value_path_is_the_oracle(oracle, tangent, phase):
    sys, fun, pp = _case(time=-0.5 if phase == PHASE_FILL else 0.0)
    cp = _coarse_grid(oracle, sys, pp)
    J, dJ, fin = tangent.run(sys, fun, cp, pp, STEPS, phase)
    want = _oracle_final(oracle, sys, fun, cp, pp, phase)
    for f in FIELDS:
        assert fin[f].tobytes() == want[f].tobytes(), f
    assert dJ.shape == (0,)


def test_tangent_directions_vs_finite_differences(oracle, tangent):
    sys, fun, pp = _case()
    cp = _coarse_grid(oracle, sys, pp)
    ref = _xrot(pp, sys)
    rng = np.random.default_rng(5)
    # directions: theta_k along each parameter (so dJ is dJ/dlog theta), then two of the state
    dsys = np.zeros(tangent.ndirs, dtype=SYSTEM_PAR)
    for k, name in enumerate(PARAMS):
        dsys[k][name] = float(sys[name])
    rmax = float(sys["rmax"])
    dpp = np.zeros((tangent.ndirs, N), dtype=PARTICLE)
    dpp[6] = state_tangent(pp, sys, dr=rng.standard_normal((N, 3)) * rmax, dphi=rng.standard_normal((N, 3)))
    dpp[7] = state_tangent(pp, sys, dv=rng.standard_normal((N, 3)) * 10.0, dw=rng.standard_normal((N, 3)) * 30.0)
    _, dJ, _ = tangent.run(sys, fun, cp, pp, STEPS, dsys=dsys, dpp=dpp)
    fd = []
    for k, name in enumerate(PARAMS):
        h = 1e-6 * float(sys[name])
        Js = []
        for sgn in (1.0, -1.0):
            s2 = sys.copy()
            s2[name] += sgn * h
            Js.append(_J(_oracle_final(oracle, s2, fun, cp, pp, PHASE_AVALANCHE), sys, ref))
        fd.append((Js[0] - Js[1]) / (2e-6))
    for k in (6, 7):
        h = 1e-6
        Js = [_J(_oracle_final(oracle, sys, fun, cp, _shift(pp, dpp[k], sgn * h), PHASE_AVALANCHE), sys, ref)
              for sgn in (1.0, -1.0)]
        fd.append((Js[0] - Js[1]) / (2 * h))
    fd = np.array(fd)
    scale = float(np.abs(fd).max())
    bad = [(k, dJ[k], fd[k]) for k in range(len(fd)) if abs(dJ[k] - fd[k]) > 1e-4 * max(abs(fd[k]), 1e-3 * scale)]
    assert not bad, list(zip(dJ, fd))
    assert sum(abs(x) > 1e-3 * scale for x in fd[:6]) >= 4   # both contact laws are exercised
