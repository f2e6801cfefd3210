"""Synthetic flume workloads in the reference's cgs units.

The benchmark configurations are stated in SI with a linear spring constant kn; the reference
parameterises its contact law by a collision time t_coll instead (avalanche_hst.cu:187-193,
stiffness per sphere contact 0.5*kappa*m_eff, force_part.cu:121).  The mapping used here:

    m_s     = (4/3) pi rho r^3                       sphere mass
    kappa   = 2 kn / m_s                             so that 0.5*kappa*m_s = kn
    t_coll  = sqrt((pi^2 + ln(e)^2) / kappa)         DataInput.dat line 12

One t_coll serves particle-particle and particle-wall contacts, as in the reference.  Clumps are
the reference's tetrahedral 4-sphere clumps (edge 2r, init_Verlet.cu:130-142).
"""
from __future__ import annotations

import math
import dataclasses
from dataclasses import dataclass

import numpy as np

from ._lib import INPUTS, PARTICLE
from .engine import (Rannew64, calculate_particle_parameters, derive_system, lattice_block, lattice_pile,
                     set_initial_velocity, sphere_centres)

HOP_WIDTH, HOP_HEIGHT, YHOP_L, YHOP_R = 15.0, 25.0, 7.5, 22.5
LFUNNEL = 70.0


@dataclass
class FlumeConfig:
    """One flume run: geometry, material and the lattice release block (cgs units)."""
    n: int
    tilt_deg: float = 35.0
    width: float = 20.0          # flume width side.y [cm]
    Lflume: float = 200.0        # flume length [cm]
    radius: float = 0.1          # sphere radius [cm]
    density: float = 2.5         # [g/cm^3]
    kn: float = 1.0e7            # linear spring constant [dyn/cm] (1e4 N/m)
    restitution: float = 0.5
    mu_pp: float = 0.5
    mu_pw: float = 0.4
    dt: float = 2.0e-6
    pitch: float = 0.4           # lattice pitch of the release block [cm]
    v0: float = 0.0              # initial speed in the reference's random directions
    seed: int = 20240613         # rannew64 seed of the orientations
    hopper_height: float | None = None
    layout: str = "lattice"      # "lattice" | "pile" | "bed" (see flume_state)
    overlap: float | None = None  # how far each clump is pressed into its support [cm]:
                                  # pile 2e-5 (default), bed 0 (default; gravity loads the layer)

    @property
    def t_coll(self) -> float:
        m_s = 4.0 / 3.0 * math.pi * self.radius ** 3 * self.density
        kappa = 2.0 * self.kn / m_s
        return math.sqrt((math.pi ** 2 + math.log(self.restitution) ** 2) / kappa)


def flume_inputs(cfg: FlumeConfig) -> np.ndarray:
    """The 16 DataInput.dat values of a configuration."""
    per_layer = int(HOP_WIDTH // cfg.pitch) ** 2
    layers = -(-cfg.n // per_layer)
    height = cfg.hopper_height if cfg.hopper_height is not None else layers * cfg.pitch * 1.25 + 1.0
    v = np.zeros((), dtype=INPUTS)
    v["npart"] = cfg.n
    v["width"], v["hopper_height"] = cfg.width, height
    v["rmin"] = v["rmax"] = cfg.radius
    v["v0"], v["dt"] = cfg.v0, cfg.dt
    v["eps_pw"] = v["eps_pp"] = cfg.restitution
    v["mu_pw"], v["mu_pp"] = cfg.mu_pw, cfg.mu_pp
    v["t_coll"], v["Lflume"], v["tilt_deg"] = cfg.t_coll, cfg.Lflume, cfg.tilt_deg
    v["ntags"], v["print_flag"] = 9, 0
    return v


def flume_system_of(cfg: FlumeConfig):
    """(system_par, Funnel) of a configuration at the moment the door opens (time 0, avalanche
    phase: side.x = xfinal, avalanche_hst.cu:607-613); tot_mass is left to the caller."""
    sys, fun = derive_system(flume_inputs(cfg))
    sys["time"] = 0.0
    sys["side"][0] = (70.0 + cfg.Lflume) * float(sys["cost"])
    return sys, fun


def flume_state(cfg: FlumeConfig):
    """(system_par, Funnel, particle array) of a clump block in the hopper at the moment the door
    opens (time 0, avalanche phase: side.x = xfinal, avalanche_hst.cu:607-613).

    layout "lattice": clumps on a cubic lattice of the given pitch inside the hopper box x in
    [0, 15], y in [7.5, 22.5], z > 25, each with a uniformly random orientation (Shoemake
    quaternion from rannew64); orientations that would overlap a placed neighbour or a hopper
    wall are redrawn.
    layout "pile": the same lattice columns and random orientations, each clump dropped onto the
    closed door (z = 25) or the clumps already placed and pressed `overlap` into its support: the
    packed pile the hopper-fill phase ends with, every resting contact carrying load.  Once the
    door is open the pile falls freely, so its contacts relax within a few tens of steps.
    layout "bed": the same packing built on the flume bed instead, in the slope frame (floor
    z' = 0, side walls y = dy2 and dy2 + width, 1 cm clear of the funnel exit and the flume end)
    and turned rigidly into the lab frame: a dense layer that gravity keeps pressed on the bed
    while it slides, the state of an avalanche in full flow.
    With v0 > 0 the velocities follow the reference's set_initial_velocity (seed 26752658)."""
    sys, fun = flume_system_of(cfg)
    pp = np.zeros(cfg.n, dtype=PARTICLE)
    pp["radius"] = cfg.radius
    pp["density"] = cfg.density
    calculate_particle_parameters(pp)
    rng = Rannew64(cfg.seed)
    top = HOP_HEIGHT + float(sys["side"][2])
    if cfg.layout == "pile":
        placed = lattice_pile(pp, (0.0, YHOP_L, HOP_HEIGHT), (HOP_WIDTH, YHOP_R, top), cfg.pitch,
                              2.0e-5 if cfg.overlap is None else cfg.overlap, rng)
    elif cfg.layout == "bed":
        dy2 = float(sys["dy2"])
        placed = lattice_pile(pp, (LFUNNEL + 1.0, dy2, 0.0), (LFUNNEL + cfg.Lflume - 1.0, dy2 + cfg.width, 1e9),
                              cfg.pitch, 0.0 if cfg.overlap is None else cfg.overlap, rng)
        slope_to_lab(pp, sys)
    else:
        placed = lattice_block(pp, (0.0, YHOP_L, HOP_HEIGHT), (HOP_WIDTH, YHOP_R, top), cfg.pitch, rng)
    if placed != cfg.n:
        raise ValueError("lattice block holds %d of %d clumps" % (placed, cfg.n))
    if cfg.v0 > 0:
        set_initial_velocity(sys, pp)
    slope_frame(pp, sys)
    sys["tot_mass"] = float(pp["mass"].sum())
    return sys, fun, pp


def slope_to_lab(pp: np.ndarray, sys: np.ndarray) -> None:
    """Turn clumps built in slope-frame coordinates into the lab frame (the inverse of
    rotate_vectors.cu:28-46: x = x' cos + z' sin, y = y', z = z' cos - x' sin), centres and
    orientation matrices alike; the sphere centres are then recomputed from them."""
    c, s = float(sys["cost"]), float(sys["sint"])
    r = pp["rr"].copy()
    pp["rr"][:, 0] = r[:, 0] * c + r[:, 2] * s
    pp["rr"][:, 2] = r[:, 2] * c - r[:, 0] * s
    mx, mz = pp["Rmatx"].copy(), pp["Rmatz"].copy()
    pp["Rmatx"] = mx * c + mz * s
    pp["Rmatz"] = mz * c - mx * s
    sphere_centres(pp)


def slope_frame(pp: np.ndarray, sys: np.ndarray) -> None:
    """Fill the slope-frame copies rrot, rrot_a..d from the lab-frame positions with the arithmetic
    of rotate_vectors.cu:28-46 (x' = x cos - z sin, y' = y, z' = x sin + z cos)."""
    c, s = float(sys["cost"]), float(sys["sint"])
    for src, dst in (("rr", "rrot"), ("rr_s", "rrot_s")):
        v = pp[src]
        out = np.empty_like(v)
        out[..., 0] = v[..., 0] * c - v[..., 2] * s
        out[..., 1] = v[..., 1]
        out[..., 2] = v[..., 0] * s + v[..., 2] * c
        pp[dst] = out


# The benchmark configurations (cgs).  FLUME_2K: 2,048 clumps, 30 deg, 40 cm x 4 cm flume;
# FLUME_262K: 262,144 clumps, 35 deg, 200 cm x 20 cm flume.
def flume_2k(**kw) -> FlumeConfig:
    kw = {"n": 2048, "tilt_deg": 30.0, "width": 4.0, "Lflume": 40.0, **kw}
    return FlumeConfig(**kw)


def flume_262k(**kw) -> FlumeConfig:
    kw = {"n": 262144, "tilt_deg": 35.0, "width": 20.0, "Lflume": 200.0, **kw}
    return FlumeConfig(**kw)


# Batched ensemble: independent flumes of the 2,048-clump geometry (40 cm x 4 cm flume) with
# uneven clump counts and their own friction, restitution and slope.
ENSEMBLE_SEED = 7340033


def ensemble_configs(nflumes: int = 256, nmin: int = 1024, nmax: int = 16384, seed: int = ENSEMBLE_SEED,
                     **kw) -> list[FlumeConfig]:
    """Per flume, five rannew64 draws in this order: clump count ~ U{nmin..nmax}, mu_pp ~
    U[0.2, 0.8], mu_pw ~ U[0.2, 0.6], restitution ~ U[0.2, 0.8], inclination ~ U[25, 40] deg.
    Flume f's orientations use seed + 1 + f.  Some draws fail the reference's admission test
    tan(tilt) >= 1.25 mu_pw (error_check.cu:58); they are kept (see `ensemble_flagged`)."""
    rng = Rannew64(seed)
    out = []
    for f in range(nflumes):
        n = nmin + min(int(rng() * (nmax - nmin + 1)), nmax - nmin)
        mu_pp = 0.2 + 0.6 * rng()
        mu_pw = 0.2 + 0.4 * rng()
        e = 0.2 + 0.6 * rng()
        tilt = 25.0 + 15.0 * rng()
        out.append(flume_2k(**{"n": n, "mu_pp": mu_pp, "mu_pw": mu_pw, "restitution": e, "tilt_deg": tilt,
                               "seed": seed + 1 + f, **kw}))
    return out


def ensemble_flagged(cfgs: list[FlumeConfig]) -> list[int]:
    """Flumes the reference's error_check would refuse (tan(tilt) < 1.25 mu_pw)."""
    return [f for f, c in enumerate(cfgs) if math.tan(math.radians(c.tilt_deg)) < 1.25 * c.mu_pw]


def ensemble_state(cfgs: list[FlumeConfig]):
    """(system_par[F], Funnel[F], particle array of every flume back to back) for an ensemble
    context; flume f's clumps carry ids [sum of earlier counts, + cfgs[f].n)."""
    states = [flume_state(c) for c in cfgs]
    sys = np.stack([s for s, _, _ in states])
    fun = np.stack([u for _, u, _ in states])
    pp = np.concatenate([p for _, _, p in states])
    return sys, fun, pp


ADJOINT_BATCH_SEED = 5242883


def adjoint_batch(cfg: FlumeConfig, samples: int = 64, seed: int = ADJOINT_BATCH_SEED):
    """A calibration batch: `samples` copies of the flume `cfg` (same clumps, same initial
    state) whose material parameters are drawn per copy from rannew64 in this order: mu_pp ~
    U[0.2, 0.8], mu_pw ~ U[0.2, 0.6], restitution ~ U[0.2, 0.8] (the ranges of the ensemble
    workload).  Returns (configs, system_par[F], Funnel[F], particle array of all copies back to
    back) for an ensemble context."""
    sys0, fun0, pp = flume_state(cfg)
    rng = Rannew64(seed)
    cfgs, syss, funs = [], [], []
    for _ in range(samples):
        mu_pp = 0.2 + 0.6 * rng()
        mu_pw = 0.2 + 0.4 * rng()
        e = 0.2 + 0.6 * rng()
        c = dataclasses.replace(cfg, mu_pp=mu_pp, mu_pw=mu_pw, restitution=e)
        s, u = flume_system_of(c)
        s["tot_mass"] = sys0["tot_mass"]
        cfgs.append(c)
        syss.append(s)
        funs.append(u)
    return cfgs, np.stack(syss), np.stack(funs), np.concatenate([pp] * samples)
