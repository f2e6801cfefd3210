"""Gradients of a flume run with respect to the configuration's material parameters, and a
torch.autograd.Function over the engine's adjoint.

The engine's adjoint (`af3d_adjoint`) returns dJ/d(kappa, gamma, mu) of system_par, for the
particle-particle and the particle-wall law.  The configuration (FlumeConfig) states the material
as (mu_pp, mu_wall, restitution e, kn); the reference derives (avalanche_hst.cu:187-193,
workloads.py)

    L = ln e,  kappa0 = 2 kn / m_s,  t_coll = sqrt((pi^2 + L^2) / kappa0),
    kappa = (pi^2 + L^2) / t_coll^2 (= kappa0),  gamma = -2 L / t_coll = -2 L sqrt(kappa0 / (pi^2 + L^2)),

for both laws alike (one t_coll and one restitution serve both), so the chain rule below maps
the six engine gradients to the four configuration gradients.
"""
from __future__ import annotations

import math

import numpy as np


def sphere_mass(cfg) -> float:
    return 4.0 / 3.0 * math.pi * cfg.radius ** 3 * cfg.density


def config_gradients(cfg, params: dict) -> dict:
    """dJ/d(mu_pp, mu_pw, restitution, kn) of a FlumeConfig from the engine's dJ/d(system_par)."""
    m_s = sphere_mass(cfg)
    kappa0 = 2.0 * cfg.kn / m_s
    L = math.log(cfg.restitution)
    q = math.pi ** 2 + L * L
    dkappa_dkn = 2.0 / m_s
    dgamma_dkappa0 = -L / math.sqrt(kappa0 * q)
    dgamma_dL = -2.0 * math.sqrt(kappa0) * math.pi ** 2 / q ** 1.5
    kb = params["kappa_pp"] + params["kappa_pw"]
    gb = params["gamma_pp"] + params["gamma_pw"]
    return {"mu_pp": params["mu_pp"], "mu_pw": params["mu_pw"],
            "restitution": gb * dgamma_dL / cfg.restitution,
            "kn": kb * dkappa_dkn + gb * dgamma_dkappa0 * dkappa_dkn}


def rotation_gradient(R: np.ndarray, R_b: np.ndarray) -> np.ndarray:
    """dJ/dphi for a small rotation R -> exp([phi]x) R, per clump, from dJ/dR (rows)."""
    # dJ = sum_ij R_b_ij ([dphi]x R)_ij;  [e_x]x R = rows (0, -R_z, R_y), ...
    gx = np.einsum("nj,nj->n", R_b[:, 2], R[:, 1]) - np.einsum("nj,nj->n", R_b[:, 1], R[:, 2])
    gy = np.einsum("nj,nj->n", R_b[:, 0], R[:, 2]) - np.einsum("nj,nj->n", R_b[:, 2], R[:, 0])
    gz = np.einsum("nj,nj->n", R_b[:, 1], R[:, 0]) - np.einsum("nj,nj->n", R_b[:, 0], R[:, 1])
    return np.stack([gx, gy, gz], axis=1)


def downslope(pp: np.ndarray, sys) -> np.ndarray:
    """x_rot = x cos(tilt) - z sin(tilt) of every clump centre (rotate_vectors.cu:28)."""
    return pp["rr"][:, 0] * float(sys["cost"]) - pp["rr"][:, 2] * float(sys["sint"])


def runout(pp: np.ndarray, sys, length: float) -> float:
    """The runout objective of af3d_set_objective on a host state: length * ln(sum m exp(x /
    length) / sum m) over the downslope positions x, evaluated about the largest x."""
    x = downslope(pp, sys)
    m = pp["mass"]
    xmax = float(np.max(x))
    return xmax + length * math.log(float(np.sum(m * np.exp((x - xmax) / length))) / float(np.sum(m)))


def flume_run_function():
    """A torch.autograd.Function over the engine's adjoint:

        J = FlumeRun.apply(r0, make_engine, steps, ckpt_every, runout)

    r0 is an (n, 3) tensor of initial clump positions; make_engine(r0 as a numpy array) returns
    an Engine with the state imported (the sphere centres placed at r0); runout is None for the
    deposit centroid or the runout length scale.  J is a scalar for a single flume, or a tensor
    of one J per flume for an ensemble.  Its gradient with respect to r0 comes from
    af3d_adjoint (the sphere centres follow r0): for an ensemble each clump's gradient is
    scaled by the incoming gradient of its own flume's J."""
    import torch

    class FlumeRun(torch.autograd.Function):
        @staticmethod
        def forward(ctx, r0, make_engine, steps, ckpt_every, runout_length=None):
            eng = make_engine(r0.detach().cpu().numpy())
            try:
                out = eng.adjoint(int(steps), int(ckpt_every), gradients=True, runout=runout_length)
                flume_of = np.repeat(np.arange(eng.nflumes), eng.flume_sizes)
                ensemble = eng.ensemble
            finally:
                eng.close()
            ctx.save_for_backward(torch.as_tensor(out["r0"], dtype=r0.dtype, device=r0.device),
                                  torch.as_tensor(flume_of, device=r0.device))
            ctx.ensemble = ensemble
            return torch.as_tensor(np.asarray(out["J"], dtype=np.float64), dtype=r0.dtype, device=r0.device)

        @staticmethod
        def backward(ctx, gJ):
            g, flume_of = ctx.saved_tensors
            scale = gJ[flume_of] if ctx.ensemble else gJ
            return g * (scale[:, None] if ctx.ensemble else scale), None, None, None, None

    return FlumeRun
