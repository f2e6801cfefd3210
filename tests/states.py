"""Seeded synthetic clump states and the reference step sequence driven through either CPU
library (the restatement or the reference built from source) -- test helpers."""
from __future__ import annotations

import numpy as np

from oracle.pyoracle import (CELL_PAR, GYR, HOP_HEIGHT, HOP_WIDTH, LFUNNEL, PARTICLE, PHASE_FILL,
                             dense_state, grid_from_bbox, make_system, mass_inertia,
                             random_rotations, rotate_slope, sphere_centres, xfinal)


def flume_system(n, tilt=35.0, width=20.0, Lflume=200.0, rmax=0.1, rmin=None, dt=2e-6, time=0.0,
                 mu_pp=0.5, mu_pw=0.4, eps=0.5, t_coll=7.3615e-5, hopper_height=80.0, side_x=None):
    """system_par for a flume workload in the reference's cgs units (avalanche phase: time >= 0 and
    side.x = xfinal unless given)."""
    sys, fun = make_system(n, width, hopper_height, rmin if rmin is not None else rmax, rmax, 10.0,
                           dt, eps, mu_pw, eps, mu_pp, t_coll, Lflume, tilt, time=time)
    sys["side"][0] = xfinal(sys) if side_x is None else side_x
    return sys, fun


def _to_lab(q, cost, sint):
    r = np.empty_like(q)
    r[:, 0] = q[:, 0] * cost + q[:, 2] * sint
    r[:, 1] = q[:, 1]
    r[:, 2] = q[:, 2] * cost - q[:, 0] * sint
    return r


def wall_state(n, seed, sys, vel=20.0, omega=50.0):
    """Clumps spread over six clusters that touch every boundary type of the avalanche phase:
    hopper walls, funnel walls, funnel corners, flume side walls and the bed, plus a dense
    free cluster.  Clusters are dense so particle contacts occur everywhere as well."""
    rng = np.random.default_rng(seed)
    rmax = float(sys["rmax"])
    cost, sint = float(sys["cost"]), float(sys["sint"])
    dy2, width = float(sys["dy2"]), float(sys["side"][1])
    tanfi = dy2 / LFUNNEL
    pitch = 0.95 * GYR * rmax
    pts = []
    k = 0
    groups = 6
    per = [n // groups + (1 if g < n % groups else 0) for g in range(groups)]

    def block(m, origin, axes=(4, 4)):
        ii = np.arange(m)
        a, b, c = ii % axes[0], (ii // axes[0]) % axes[1], ii // (axes[0] * axes[1])
        return origin + np.stack([a, b, c], 1) * pitch + (rng.random((m, 3)) - 0.5) * 0.15 * pitch

    # 0: hopper corner (x~0, y~7.5, z~25) and 1: opposite hopper corner (x~15, y~22.5)
    pts.append(block(per[0], np.array([0.2 * rmax, 7.5 + 0.2 * rmax, HOP_HEIGHT + 0.25 * rmax])))
    o = np.array([HOP_WIDTH - 0.2 * rmax, 22.5 - 0.2 * rmax, HOP_HEIGHT + 0.3 * rmax])
    b = block(per[1], np.zeros(3))
    pts.append(o - b)
    # 2: funnel walls, in the slope frame near y = x tanfi, then rotated to the lab frame
    m = per[2]
    xr = 20.0 + rng.random(m) * 40.0
    side = rng.random(m) < 0.5
    yr = np.where(side, xr * tanfi + (rng.random(m) - 0.3) * 1.2 * rmax,
                  30.0 - xr * tanfi - (rng.random(m) - 0.3) * 1.2 * rmax)
    zr = 0.8 * rmax + rng.random(m) * 3 * rmax
    pts.append(_to_lab(np.stack([xr, yr, zr], 1), cost, sint))
    # 3: funnel corners, x_rot ~ 70, y ~ dy2 or dy2 + width
    m = per[3]
    xr = LFUNNEL + (rng.random(m) - 0.5) * 4 * rmax
    side = rng.random(m) < 0.5
    yr = np.where(side, dy2 + (rng.random(m) - 0.5) * 3 * rmax, dy2 + width + (rng.random(m) - 0.5) * 3 * rmax)
    zr = 1.0 * rmax + (np.arange(m) // 2) * pitch + rng.random(m) * 0.2 * rmax
    pts.append(_to_lab(np.stack([xr, yr, zr], 1), cost, sint))
    # 4: flume side walls and bed, x_rot in (75, 70 + L)
    m = per[4]
    xr = 75.0 + rng.random(m) * (float(sys["Lflume"]) - 10.0)
    side = rng.random(m) < 0.5
    yr = np.where(side, dy2 + 0.5 * rmax + rng.random(m) * 1.5 * rmax,
                  dy2 + width - 0.5 * rmax - rng.random(m) * 1.5 * rmax)
    zr = 0.6 * rmax + rng.random(m) * 2.5 * rmax
    pts.append(_to_lab(np.stack([xr, yr, zr], 1), cost, sint))
    # 5: a dense block resting on the bed mid-flume
    m = per[5]
    base = _to_lab(np.array([[100.0, dy2 + width / 2, 1.2 * rmax]]), cost, sint)[0]
    pts.append(block(m, base, axes=(5, 5)))

    r = np.concatenate(pts)[:n]
    pp = np.zeros(n, dtype=PARTICLE)
    pp["radius"] = rmax
    pp["density"] = 2.5
    mass_inertia(pp)
    pp["rr"] = r
    R = random_rotations(rng, n)
    pp["Rmatx"], pp["Rmaty"], pp["Rmatz"] = R[:, 0], R[:, 1], R[:, 2]
    pp["vv"] = (rng.random((n, 3)) - 0.5) * 2 * vel
    pp["ww"] = (rng.random((n, 3)) - 0.5) * 2 * omega
    sphere_centres(pp)
    rotate_slope(pp, sys)
    return pp


def grid_from_state(pp, sys, ntags, lib):
    cp = np.zeros((), dtype=CELL_PAR)
    cp["ntags"] = ntags
    hi, lo = lib.cell_dim(pp, sys)
    cp["rr_max"], cp["rr_min"] = hi, lo
    grid_from_bbox(cp, sys)
    return cp


class Work:
    """Force, torque, acceleration and cell buffers of one CPU run (reference layout)."""

    def __init__(self, n, cp):
        self.F = np.zeros((n, 3))
        self.T = np.zeros((n, 3))
        self.a_i = np.zeros((n, 3))
        self.al_i = np.zeros((n, 3))
        self.a_f = np.zeros((n, 3))
        self.al_f = np.zeros((n, 3))
        self.resize(cp)

    def resize(self, cp):
        self.cell_vec = np.full(max(1, int(cp["ntot"])), -1, dtype=np.int64)
        self.nocup = np.zeros(max(1, int(cp["ncell3"])), dtype=np.int32)


def run_forces(lib, sys, fun, cp, pp, w, phase, variant=0):
    """clear_forces, cells and every force routine of one phase in the reference's order, then
    get_accel into a_f (avalanche_hst.cu:444-464 fill, :678-707 avalanche)."""
    lib.clear_forces(sys, w.F, w.T)
    lib.clear_cell(cp, w.cell_vec)
    lib.clear_ocup(cp, w.nocup)
    st = lib.cell_locate(cp, sys, pp, w.nocup, w.cell_vec)
    assert st == 0, st
    if phase == PHASE_FILL:
        for s in range(1, 17):
            lib.force_part(w.F, w.T, w.cell_vec, w.nocup, pp, sys, cp, s, variant)
        for nw in range(3):
            lib.force_hop(w.F, w.T, sys, pp, nw)
    else:
        for nw in range(3):
            lib.force_hop(w.F, w.T, sys, pp, nw)
        lib.force_funnel(w.F, w.T, sys, pp, fun)
        lib.force_fcorners(w.F, w.T, sys, fun, pp)
        lib.force_walls(w.F, w.T, sys, pp)
        for s in range(1, 17):
            lib.force_part(w.F, w.T, w.cell_vec, w.nocup, pp, sys, cp, s, variant)
        lib.force_flume(w.F, w.T, sys, pp)
    lib.get_accel(w.F, w.T, w.a_f, w.al_f, sys, pp)


def run_step(lib, sys, fun, cp, pp, w, phase, variant=0):
    """One full step of the reference loop (init_Verlet ... finish_Verlet, swap)."""
    lib.init_verlet(w.a_i, w.al_i, sys, pp)
    sys["time"] = float(sys["time"]) + float(sys["dt"])
    if phase != PHASE_FILL:
        lib.rotate_vectors(pp, sys)
    run_forces(lib, sys, fun, cp, pp, w, phase, variant)
    lib.finish_verlet(w.a_i, w.al_i, w.a_f, w.al_f, sys, pp)
    w.a_i, w.a_f = w.a_f, w.a_i
    w.al_i, w.al_f = w.al_f, w.al_i


def sorted_order(cp, w):
    """(cell, id)-sorted clump ids and their cells from the reference's slot table."""
    ntags = int(cp["ntags"])
    ids, cells = [], []
    for c in np.nonzero(w.nocup)[0]:
        k = int(w.nocup[c])
        ids.extend(w.cell_vec[c * ntags:c * ntags + k].tolist())
        cells.extend([int(c)] * k)
    return np.array(ids, dtype=np.int64), np.array(cells, dtype=np.int64)
