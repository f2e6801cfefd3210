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
    size_spread: float = 0.0     # per-clump size factor ~ U[1 - spread, 1 + spread] (polydisperse)
    ntags: int = 9               # DataInput.dat line 15: slots per cell (at most ntags - 1 clumps)
    layout: str = "lattice"      # "lattice" | "pile" | "bed" (see flume_state); "funnel" (see funnel_state)
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
    v["rmin"] = cfg.radius * (1.0 - cfg.size_spread)
    v["rmax"] = cfg.radius * (1.0 + cfg.size_spread)
    v["v0"], v["dt"] = cfg.v0, cfg.dt
    v["eps_pw"] = v["eps_pp"] = cfg.restitution
    v["mu_pw"], v["mu_pp"] = cfg.mu_pw, cfg.mu_pp
    v["t_coll"], v["Lflume"], v["tilt_deg"] = cfg.t_coll, cfg.Lflume, cfg.tilt_deg
    v["ntags"], v["print_flag"] = cfg.ntags, 0
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
    z' = 0, side walls y = dy2 and dy2 + width, 1 cm clear of the funnel exit and of the flume
    end, see bed_pile) and turned rigidly into the lab frame: a dense layer that gravity keeps
    pressed on the bed while it slides, the state of an avalanche in full flow.
    With v0 > 0 the velocities follow the reference's set_initial_velocity (seed 26752658).
    layout "funnel": see funnel_state."""
    if cfg.layout == "funnel":
        return funnel_state(cfg)
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
        placed = bed_pile(pp, sys, (LFUNNEL + 1.0, dy2, 0.0), (LFUNNEL + cfg.Lflume - 1.0, dy2 + cfg.width, 1e9),
                          cfg.pitch, 0.0 if cfg.overlap is None else cfg.overlap, rng)
    else:
        placed = lattice_block(pp, (0.0, YHOP_L, HOP_HEIGHT), (HOP_WIDTH, YHOP_R, top), cfg.pitch, rng)
    if placed != cfg.n:
        raise ValueError("lattice block holds %d of %d clumps" % (placed, cfg.n))
    if cfg.v0 > 0:
        set_initial_velocity(sys, pp)
    slope_frame(pp, sys)
    sys["tot_mass"] = float(pp["mass"].sum())
    return sys, fun, pp


def size_factors(cfg: FlumeConfig, rng: Rannew64) -> np.ndarray:
    """Per-clump size factors 1 + spread (2u - 1), u from rannew64 in clump order (all ones when
    the configuration is monodisperse)."""
    if cfg.size_spread <= 0.0:
        return np.ones(cfg.n)
    return np.array([1.0 + cfg.size_spread * (2.0 * rng() - 1.0) for _ in range(cfg.n)])


def funnel_state(cfg: FlumeConfig):
    """(system_par, Funnel, particle array) of a hopper discharging through the funnel onto the
    flume, at the moment the door opens (time 0, avalanche phase, side.x = xfinal): every
    boundary routine of the reference has clumps to act on.

    Each clump is scaled by its own factor (sphere radius and tetrahedron edge together, mass and
    inertia from calculate_particle_parameters' formulas), drawn from rannew64 before the
    orientations.  The clumps are built as lattice piles (`lattice_pile`, each clump lowered
    onto the floor or the clumps already placed, random orientations kept inside the box walls):
      * the first half in the hopper box x in [0, 15], y in [7.5, 22.5] on the door plane z = 25
        (lab frame): the pile the filling phase ends with, falling once the door is open and
        loading the hopper's side walls;
      * the second half on the bed in the slope frame: the funnel section x' in [1, 69] cut into
        strips 4 cm long, each strip's box spanning y between the converging funnel walls at its
        narrow end, and the flume x' in [71, 70 + L - 1] between its side walls (see bed_pile);
        the flume section gets at most 10 clumps per lattice column, the funnel strips the rest
        in proportion to their areas, then the layer is turned rigidly into the lab frame.  The layer touches the funnel walls, the funnel
        corners, the flume side walls and the bed.
    A strip's clumps keep every sphere inside the strip's box, so clumps of neighbouring strips
    do not overlap; the hopper pile lies upslope of the bed (x' <= 0.5)."""
    sys, fun = flume_system_of(cfg)
    pp = np.zeros(cfg.n, dtype=PARTICLE)
    rng = Rannew64(cfg.seed)
    pp["radius"] = cfg.radius * size_factors(cfg, rng)
    pp["density"] = cfg.density
    calculate_particle_parameters(pp)
    overlap = 0.0 if cfg.overlap is None else cfg.overlap
    n_hop = cfg.n // 2
    top = HOP_HEIGHT + float(sys["side"][2])
    hop = pp[:n_hop].copy()
    placed = lattice_pile(hop, (0.0, YHOP_L, HOP_HEIGHT), (HOP_WIDTH, YHOP_R, top), cfg.pitch, overlap, rng)
    if placed != n_hop:
        raise ValueError("the hopper holds %d of %d clumps below its top" % (placed, n_hop))
    pp[:n_hop] = hop
    dy2 = float(sys["dy2"])
    tanfi = dy2 / LFUNNEL
    boxes = []
    x0 = 1.0
    while x0 < LFUNNEL - 1.0 - 1e-9:
        x1 = min(x0 + 4.0, LFUNNEL - 1.0)
        boxes.append(((x0, x1 * tanfi, 0.0), (x1, 30.0 - x1 * tanfi, 1e9)))
        x0 = x1
    boxes.append(((LFUNNEL + 1.0, dy2, 0.0), (LFUNNEL + cfg.Lflume - 1.0, dy2 + cfg.width, 1e9)))
    cols = np.array([np.floor((hi[0] - lo[0]) / cfg.pitch) * np.floor((hi[1] - lo[1]) / cfg.pitch)
                     for lo, hi in boxes])
    n_bed = cfg.n - n_hop
    # the flume section holds at most 10 clumps per column (a layer a few cm deep; deeper, its
    # top would reach past the flume end), the funnel strips the rest in proportion to their areas
    flume_share = min(int(10 * cols[-1]), int(n_bed * cols[-1] / cols.sum()))
    share = np.floor((n_bed - flume_share) * cols / cols[:-1].sum()).astype(np.int64)
    share[-1] = flume_share
    share[np.argmax(cols[:-1])] += n_bed - int(share.sum())
    start = n_hop
    for (lo, hi), m in zip(boxes, share):
        part = pp[start:start + m].copy()
        if bed_pile(part, sys, lo, hi, cfg.pitch, overlap, rng) != m:
            raise ValueError("a bed strip holds fewer clumps than its share")
        pp[start:start + m] = part
        start += m
    slope_frame(pp, sys)
    sys["tot_mass"] = float(pp["mass"].sum())
    return sys, fun, pp


def bed_pile(pp: np.ndarray, sys: np.ndarray, lo, hi, pitch: float, overlap: float, rng: Rannew64,
             margin: float = 1.0) -> int:
    """lattice_pile on the bed in the slope frame (box lo..hi in slope-frame coordinates), turned
    into the lab frame.  The box's downslope end is pulled back, and the pile built again from the
    same generator state, until every clump centre lies `margin` upslope of the flume end x =
    side.x in the lab frame: the top of a deep layer reaches farther downslope in the lab frame
    than its foot, and a clump past side.x is removed at the first step (init_Verlet.cu:29-33).
    Returns the clumps placed."""
    c, s = float(sys["cost"]), float(sys["sint"])
    limit = float(sys["side"][0]) - margin
    x_hi = float(hi[0])
    for _ in range(16):
        part = pp.copy()
        g = rng.clone()
        placed = lattice_pile(part, lo, (x_hi, hi[1], hi[2]), pitch, overlap, g)
        over = float(np.max(part["rr"][:placed, 0] * c + part["rr"][:placed, 2] * s)) - limit if placed else 0.0
        if over <= 0.0 or placed < len(pp):
            pp[:] = part
            rng.assign(g)
            slope_to_lab(pp, sys)
            return placed
        x_hi -= over / c + pitch
    raise ValueError("the bed layer does not fit upslope of the flume end")


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


# FUNNEL_524K: 524,288 polydisperse clumps (size factor U[0.8, 1.2]) in the reference's hopper,
# funnel and 40 cm x 4 cm flume at 30 deg (the 2,048-clump geometry), half in the hopper and half
# on the funnel and flume bed (funnel_state); the lattice pitch 4.5 mm; hopper 100 cm high.  The
# densest cells of this packing hold 8 of the smaller clumps, the most 9 slots allow, so the
# cells get 16 slots.
def funnel_524k(**kw) -> FlumeConfig:
    kw = {"n": 524288, "tilt_deg": 30.0, "width": 4.0, "Lflume": 40.0, "size_spread": 0.2, "pitch": 0.45,
          "hopper_height": 100.0, "layout": "funnel", "seed": 3145739, "ntags": 16, **kw}
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
