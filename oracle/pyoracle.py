"""ctypes bindings for the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Imported by ``tests/`` (the parity checker), by ``__graft_entry__.smoke()``
and by ``bench.py``'s CPU-baseline leg; never by the product package.

``Oracle`` wraps ``oracle/liboracle_af3d.so`` (the restatement) and
``Reference`` wraps ``oracle/_ref/libaf3d_ref.so`` (the reference's own
routines compiled from source, only where the reference tree exists).  Both
expose the same per-routine methods taking numpy arrays of the structured
dtypes below, whose layouts equal the reference's structs (cabecera.hu:34-112).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

VEC3 = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8")])

SYSTEM_PAR = np.dtype([("npart", "<i8")] + [(f, "<f8") for f in (
    "dt", "hdt", "rmin", "rmax", "v0", "time", "eps_pp", "eps_pw", "kappa_pp", "kappa_pw",
    "gamma_pp", "gamma_pw", "mu_pp", "mu_pw", "t_coll", "tot_mass", "tilt", "xhopper", "Lflume",
    "gyr_max", "fr_fact_pp", "fr_fact_pw", "sint", "cost", "sintg", "costg", "xfunnel", "dy2")]
    + [("side", "<f8", (3,))])

FUNNEL = np.dtype([("sinfi", "<f8"), ("cosfi", "<f8"), ("tanfi", "<f8")])

PARTICLE = np.dtype([
    ("radius", "<f8"), ("mass", "<f8"), ("density", "<f8"), ("moment_of_inertia", "<f8", (3,)),
    ("rr_s", "<f8", (4, 3)), ("rrot_s", "<f8", (4, 3)), ("rr", "<f8", (3,)), ("rrot", "<f8", (3,)),
    ("vv", "<f8", (3,)), ("ww", "<f8", (3,)), ("Rmatx", "<f8", (3,)), ("Rmaty", "<f8", (3,)),
    ("Rmatz", "<f8", (3,))])

CELL_PAR = np.dtype([
    ("ntags", "<i8"), ("ncell3", "<i8"), ("ncell", "<i8", (3,)), ("ntot", "<i8"),
    ("cell_side", "<f8", (3,)), ("cs_inv", "<f8", (3,)), ("rr_max", "<f8", (3,)),
    ("rr_min", "<f8", (3,)), ("length", "<f8", (3,))])

assert SYSTEM_PAR.itemsize == 256 and PARTICLE.itemsize == 408 and CELL_PAR.itemsize == 168

FRICTION_HST, FRICTION_DEV = 0, 1
PHASE_FILL, PHASE_AVALANCHE = 0, 1

# cabecera.hu:5-19
PI = 3.1415926535897932
GYR = 4.4494897427831781
SPH_FACT = 4.188790204786391
ROOT2 = 1.414213562373095
LFUNNEL, YFUNNEL, HOP_WIDTH, HOP_HEIGHT = 70.0, 30.0, 15.0, 25.0


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def vec3_array(n: int) -> np.ndarray:
    return np.zeros((n, 3), dtype=np.float64)


class _Work(C.Structure):
    _fields_ = [("force", C.c_void_p), ("torque", C.c_void_p), ("acc_i", C.c_void_p),
                ("anga_i", C.c_void_p), ("acc_f", C.c_void_p), ("anga_f", C.c_void_p),
                ("cell_vec", C.c_void_p), ("nocup_vec", C.c_void_p),
                ("cell_vec_cap", C.c_long), ("nocup_cap", C.c_long)]


class Oracle:
    """The C restatement (oracle/af3d_oracle.c)."""

    def __init__(self, path: str | None = None):
        if path is None:
            from oracle import build as _b
            path = _b.build_oracle()
        self.lib = C.CDLL(path)
        L = self.lib
        L.orc_cell_locate.restype = C.c_int
        L.orc_step.restype = C.c_int
        L.orc_forces.restype = C.c_int
        L.orc_contact_pairs.restype = C.c_long
        L.orc_contact_pairs.argtypes = [C.c_void_p, C.c_long] + [C.c_void_p] * 5 + [C.c_int]
        for name in ("orc_force_hop",):
            getattr(L, name).argtypes = [C.c_void_p] * 4 + [C.c_int]
        L.orc_force_part.argtypes = [C.c_void_p] * 7 + [C.c_int, C.c_int]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_step.argtypes = [C.c_void_p] * 4 + [C.POINTER(_Work), C.c_int, C.c_int]
        L.orc_forces.argtypes = [C.c_void_p] * 4 + [C.POINTER(_Work), C.c_int, C.c_int]

    def set_threads(self, n: int) -> None:
        self.lib.orc_set_threads(int(n))

    # -- per-routine (same argument order as the reference routines) --
    def init_verlet(self, acc, anga, sys, pp):
        self.lib.orc_init_verlet(_p(acc), _p(anga), _p(sys), _p(pp))

    def rotate_vectors(self, pp, sys):
        self.lib.orc_rotate_vectors(_p(pp), _p(sys))

    def clear_forces(self, sys, f, t):
        self.lib.orc_clear_forces(_p(sys), _p(f), _p(t))

    def clear_cell(self, cp, cell_vec):
        self.lib.orc_clear_cell(_p(cp), _p(cell_vec))

    def clear_ocup(self, cp, nocup):
        self.lib.orc_clear_ocup(_p(cp), _p(nocup))

    def cell_locate(self, cp, sys, pp, nocup, cell_vec) -> int:
        return self.lib.orc_cell_locate(_p(cp), _p(sys), _p(pp), _p(nocup), _p(cell_vec))

    def force_hop(self, f, t, sys, pp, nw):
        self.lib.orc_force_hop(_p(f), _p(t), _p(sys), _p(pp), int(nw))

    def force_funnel(self, f, t, sys, pp, fun):
        self.lib.orc_force_funnel(_p(f), _p(t), _p(sys), _p(pp), _p(fun))

    def force_fcorners(self, f, t, sys, fun, pp):
        self.lib.orc_force_fcorners(_p(f), _p(t), _p(sys), _p(fun), _p(pp))

    def force_walls(self, f, t, sys, pp):
        self.lib.orc_force_walls(_p(f), _p(t), _p(sys), _p(pp))

    def force_part(self, f, t, cell_vec, nocup, pp, sys, cp, sph_id, variant=FRICTION_HST):
        self.lib.orc_force_part(_p(f), _p(t), _p(cell_vec), _p(nocup), _p(pp), _p(sys), _p(cp),
                                int(sph_id), int(variant))

    def force_flume(self, f, t, sys, pp):
        self.lib.orc_force_flume(_p(f), _p(t), _p(sys), _p(pp))

    def get_accel(self, f, t, a, al, sys, pp):
        self.lib.orc_get_accel(_p(f), _p(t), _p(a), _p(al), _p(sys), _p(pp))

    def finish_verlet(self, ai, ali, af, alf, sys, pp):
        self.lib.orc_finish_verlet(_p(ai), _p(ali), _p(af), _p(alf), _p(sys), _p(pp))

    def cell_dim(self, pp, sys):
        hi, lo = np.zeros(3), np.zeros(3)
        self.lib.orc_cell_dim(_p(hi), _p(lo), _p(pp), _p(sys))
        return hi, lo

    def grid_from_bbox(self, cp, sys):
        self.lib.orc_grid_from_bbox(_p(cp), _p(sys))

    def contact_pairs(self, cell_vec, nocup, pp, sys, cp, active=False) -> np.ndarray:
        cap = 1 << 16
        while True:
            out = np.zeros((cap, 3), dtype=np.int64)
            n = self.lib.orc_contact_pairs(_p(out), cap, _p(cell_vec), _p(nocup), _p(pp), _p(sys),
                                           _p(cp), int(bool(active)))
            if n <= cap:
                return out[:n].copy()
            cap = int(n)


class Reference:
    """The reference's own host routines compiled from source (oracle/_ref/libaf3d_ref.so)."""

    def __init__(self, path: str | None = None):
        if path is None:
            from oracle import build as _b
            path = _b.build_ref()
            if path is None:
                raise FileNotFoundError("reference tree absent: oracle/_ref cannot be built")
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_force_hop_hst.argtypes = [C.c_void_p] * 4 + [C.c_int]
        L.ref_force_part_hst.argtypes = [C.c_void_p] * 7 + [C.c_int]
        L.ref_rannew64.restype = C.c_double
        L.ref_rannew64.argtypes = [C.c_void_p]
        L.ref_error_check.restype = C.c_int
        for nm in ("ref_sizeof_particle", "ref_sizeof_system_par", "ref_sizeof_cell_par"):
            getattr(L, nm).restype = C.c_long

    def init_verlet(self, acc, anga, sys, pp):
        self.lib.ref_init_Verlet_hst(_p(acc), _p(anga), _p(sys), _p(pp))

    def rotate_vectors(self, pp, sys):
        self.lib.ref_rotate_vectors_hst(_p(pp), _p(sys))

    def clear_forces(self, sys, f, t):
        self.lib.ref_clear_forces_hst(_p(sys), _p(f), _p(t))

    def clear_cell(self, cp, cell_vec):
        self.lib.ref_clear_cell_hst(_p(cp), _p(cell_vec))

    def clear_ocup(self, cp, nocup):
        self.lib.ref_clear_ocup_hst(_p(cp), _p(nocup))

    def cell_locate(self, cp, sys, pp, nocup, cell_vec) -> int:
        self.lib.ref_cell_locate_hst(_p(cp), _p(sys), _p(pp), _p(nocup), _p(cell_vec))
        return 0

    def force_hop(self, f, t, sys, pp, nw):
        self.lib.ref_force_hop_hst(_p(f), _p(t), _p(sys), _p(pp), int(nw))

    def force_funnel(self, f, t, sys, pp, fun):
        self.lib.ref_force_funnel_hst(_p(f), _p(t), _p(sys), _p(pp), _p(fun))

    def force_fcorners(self, f, t, sys, fun, pp):
        self.lib.ref_force_fcorners_hst(_p(f), _p(t), _p(sys), _p(fun), _p(pp))

    def force_walls(self, f, t, sys, pp):
        self.lib.ref_force_walls_hst(_p(f), _p(t), _p(sys), _p(pp))

    def force_part(self, f, t, cell_vec, nocup, pp, sys, cp, sph_id, variant=FRICTION_HST):
        assert variant == FRICTION_HST, "the reference host routine is the HST variant"
        self.lib.ref_force_part_hst(_p(f), _p(t), _p(cell_vec), _p(nocup), _p(pp), _p(sys), _p(cp),
                                    int(sph_id))

    def force_flume(self, f, t, sys, pp):
        self.lib.ref_force_flume_hst(_p(f), _p(t), _p(sys), _p(pp))

    def get_accel(self, f, t, a, al, sys, pp):
        self.lib.ref_get_accel_hst(_p(f), _p(t), _p(a), _p(al), _p(sys), _p(pp))

    def finish_verlet(self, ai, ali, af, alf, sys, pp):
        self.lib.ref_finish_Verlet_hst(_p(ai), _p(ali), _p(af), _p(alf), _p(sys), _p(pp))

    def cell_dim(self, pp, sys):
        hi, lo = np.zeros(3), np.zeros(3)
        self.lib.ref_cell_dim(_p(hi), _p(lo), _p(pp), _p(sys))
        return hi, lo

    def error_check(self, sys) -> int:
        buf = C.create_string_buffer(256)
        return self.lib.ref_error_check(_p(sys), buf)

    def rannew64(self, idum: np.ndarray) -> float:
        return self.lib.ref_rannew64(_p(idum))


# ----------------------------------------------------------------------------------------------
# Test-state helpers (numpy; follow the reference's start-up arithmetic)
# ----------------------------------------------------------------------------------------------

def make_system(npart, width, hopper_height, rmin, rmax, v0, dt, eps_pw, mu_pw, eps_pp, mu_pp,
                t_coll, Lflume, tilt_deg, time=0.0, side_x=None):
    """system_par and Funnel derived as avalanche_hst.cu:84-102 and :187-195 derive them."""
    import math
    s = np.zeros((), dtype=SYSTEM_PAR)
    s["npart"] = npart
    s["side"] = (HOP_WIDTH, width, hopper_height)
    s["rmin"], s["rmax"], s["v0"], s["dt"] = rmin, rmax, v0, dt
    s["eps_pw"], s["mu_pw"], s["eps_pp"], s["mu_pp"] = eps_pw, mu_pw, eps_pp, mu_pp
    s["t_coll"], s["Lflume"] = t_coll, Lflume
    s["time"] = time
    s["hdt"] = 0.5 * dt
    tilt = tilt_deg * (PI / 180.0)
    s["tilt"] = tilt
    s["gyr_max"] = GYR * rmax
    s["sint"] = math.sin(tilt)
    s["cost"] = math.cos(tilt)
    s["sintg"] = 981.0 * s["sint"]
    s["costg"] = 981.0 * s["cost"]
    s["xfunnel"] = LFUNNEL * s["cost"]
    s["dy2"] = 0.5 * (YFUNNEL - width)
    aux0 = PI / t_coll
    aux1 = math.log(eps_pp) / t_coll
    s["gamma_pp"] = -2.0 * math.log(eps_pp) / t_coll
    s["kappa_pp"] = aux0 * aux0 + aux1 * aux1
    aux1 = math.log(eps_pw) / t_coll
    s["gamma_pw"] = -2.0 * math.log(eps_pw) / t_coll
    s["kappa_pw"] = aux0 * aux0 + aux1 * aux1
    s["fr_fact_pp"] = mu_pp / 1.0e12
    s["fr_fact_pw"] = mu_pw / 1.0e12
    if side_x is not None:
        s["side"][0] = side_x
    f = np.zeros((), dtype=FUNNEL)
    dy2 = float(s["dy2"])
    hip = math.sqrt(dy2 * dy2 + LFUNNEL * LFUNNEL)
    f["sinfi"], f["cosfi"], f["tanfi"] = dy2 / hip, LFUNNEL / hip, dy2 / LFUNNEL
    return s, f


def xfinal(sys) -> float:
    """avalanche_hst.cu:116."""
    return (LFUNNEL + float(sys["Lflume"])) * float(sys["cost"])


def sphere_centres(pp: np.ndarray) -> None:
    """Sphere centres from rr and R with init_Verlet.cu:130-142's arithmetic."""
    pos = pp["radius"] / ROOT2
    r = pp["rr"]
    Rx, Ry, Rz = pp["Rmatx"], pp["Rmaty"], pp["Rmatz"]
    s = pp["rr_s"]
    for k, (R) in enumerate((Rx, Ry, Rz)):
        a, b, c = R[:, 0], R[:, 1], R[:, 2]
        s[:, 0, k] = r[:, k] + pos * ((a + b) + c)
        s[:, 1, k] = r[:, k] + pos * ((a - b) - c)
        s[:, 2, k] = r[:, k] + pos * ((-a - b) + c)
        s[:, 3, k] = r[:, k] + pos * ((-a + b) - c)
    pp["rr_s"] = s


def rotate_slope(pp: np.ndarray, sys) -> None:
    """rotate_vectors.cu:28-46."""
    c, s = float(sys["cost"]), float(sys["sint"])

    def rot(v):
        out = np.empty_like(v)
        out[..., 0] = v[..., 0] * c - v[..., 2] * s
        out[..., 1] = v[..., 1]
        out[..., 2] = v[..., 0] * s + v[..., 2] * c
        return out
    pp["rrot"] = rot(pp["rr"])
    pp["rrot_s"] = rot(pp["rr_s"])


def mass_inertia(pp: np.ndarray) -> None:
    """calculate_particle_parameters.cu:19-37 (host version)."""
    aux1 = 4.0 * PI / 3.0
    aux2 = 112.0 * PI / 15.0
    rad = pp["radius"]
    rad3 = rad * rad * rad
    rad5 = rad3 * rad * rad
    pp["mass"] = 4.0 * aux1 * rad3 * pp["density"]
    I = aux2 * pp["density"] * rad5
    pp["moment_of_inertia"] = np.stack([I, I, I], axis=1)


def random_rotations(rng: np.random.Generator, n: int) -> np.ndarray:
    """Uniform random rotation matrices (rows), from uniform unit quaternions (Shoemake)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    w, x = a * np.sin(2 * PI * u2), a * np.cos(2 * PI * u2)
    y, z = b * np.sin(2 * PI * u3), b * np.cos(2 * PI * u3)
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z); R[:, 0, 1] = 2 * (x * y - z * w); R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w); R[:, 1, 1] = 1 - 2 * (x * x + z * z); R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w); R[:, 2, 1] = 2 * (y * z + x * w); R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def grid_for(pp: np.ndarray, sys, ntags: int, lib) -> np.ndarray:
    """cell_par as avalanche_hst.cu:311-333 computes it (cell_dim + derivation)."""
    cp = np.zeros((), dtype=CELL_PAR)
    cp["ntags"] = ntags
    hi, lo = lib.cell_dim(pp, sys)
    cp["rr_max"], cp["rr_min"] = hi, lo
    grid_from_bbox(cp, sys)
    return cp


def grid_from_bbox(cp, sys) -> None:
    """avalanche_hst.cu:314-333 in numpy scalar arithmetic (float32 0.05f promoted, :115)."""
    dist = GYR + float(np.float32(0.05))
    rmax = float(sys["rmax"])
    length = cp["rr_max"] - cp["rr_min"]
    cp["length"] = length
    n = np.array([int(float(length[i]) / (dist * rmax)) for i in range(3)], dtype=np.int64)
    cp["ncell"] = n
    side = np.array([float(length[i]) / float(n[i]) for i in range(3)])
    cp["cell_side"] = side
    cp["cs_inv"] = np.array([1.0 / side[i] for i in range(3)])
    cp["ncell3"] = int(n[0] * n[1] * n[2])
    cp["ntot"] = int(cp["ncell3"]) * int(cp["ntags"])


def dense_state(n: int, seed: int, sys, pitch_factor: float = 0.85, box=(0.0, 7.5, 25.0),
                per_row=None, vel=10.0, omega=30.0, polydisperse=0.0, density=2.6, removed_frac=0.0):
    """A random dense clump state for parity tests: a jittered cubic lattice whose pitch is
    pitch_factor times the clump bounding diameter (so neighbouring clumps overlap often), random
    orientations, velocities and spins.  Sphere centres and slope-frame copies follow the
    reference's arithmetic."""
    rng = np.random.default_rng(seed)
    rmax = float(sys["rmax"])
    pp = np.zeros(n, dtype=PARTICLE)
    scale = 1.0 - polydisperse * rng.random(n) if polydisperse else np.ones(n)
    pp["radius"] = rmax * scale
    pp["density"] = density
    mass_inertia(pp)
    pitch = pitch_factor * GYR * rmax
    if per_row is None:
        per_row = max(1, int(round(n ** (1.0 / 3.0))))
    idx = np.arange(n)
    i, j, k = idx % per_row, (idx // per_row) % per_row, idx // (per_row * per_row)
    base = np.stack([box[0] + (i + 0.6) * pitch, box[1] + (j + 0.6) * pitch,
                     box[2] + (k + 0.6) * pitch], axis=1)
    pp["rr"] = base + (rng.random((n, 3)) - 0.5) * 0.1 * pitch
    R = random_rotations(rng, n)
    pp["Rmatx"], pp["Rmaty"], pp["Rmatz"] = R[:, 0], R[:, 1], R[:, 2]
    pp["vv"] = (rng.random((n, 3)) - 0.5) * 2 * vel
    pp["ww"] = (rng.random((n, 3)) - 0.5) * 2 * omega
    sphere_centres(pp)
    rotate_slope(pp, sys)
    return pp


class OracleRun:
    """A whole CPU run driven in C by orc_forces / orc_step (the reference's step sequence,
    including time += dt and the acceleration swap), with the cell grid of cell_dim."""

    def __init__(self, oracle: Oracle, sys, fun, pp, ntags=9, cp=None, acc=None, anga=None):
        self.o = oracle
        self.sys = np.array(sys, dtype=SYSTEM_PAR).copy()
        self.fun = np.array(fun, dtype=FUNNEL).copy()
        self.pp = np.ascontiguousarray(pp, dtype=PARTICLE).copy()
        n = len(self.pp)
        self.bufs = {k: np.zeros((n, 3)) for k in ("F", "T", "a0", "al0", "a1", "al1")}
        if acc is not None:
            self.bufs["a0"][:] = acc
        if anga is not None:
            self.bufs["al0"][:] = anga
        self.w = _Work()
        for f, k in (("force", "F"), ("torque", "T"), ("acc_i", "a0"), ("anga_i", "al0"),
                     ("acc_f", "a1"), ("anga_f", "al1")):
            setattr(self.w, f, self.bufs[k].ctypes.data)
        self.ntags = ntags
        if cp is None:
            cp = np.zeros((), dtype=CELL_PAR)
            cp["ntags"] = ntags
            hi, lo = oracle.cell_dim(self.pp, self.sys)
            cp["rr_max"], cp["rr_min"] = hi, lo
            oracle.grid_from_bbox(cp, self.sys)
        self.set_grid(cp)

    def set_grid(self, cp):
        self.cp = np.array(cp, dtype=CELL_PAR).copy()
        self.cell_vec = np.full(max(1, int(self.cp["ntot"])), -1, dtype=np.int64)
        self.nocup = np.zeros(max(1, int(self.cp["ncell3"])), dtype=np.int32)
        self.w.cell_vec = self.cell_vec.ctypes.data
        self.w.nocup_vec = self.nocup.ctypes.data
        self.w.cell_vec_cap = len(self.cell_vec)
        self.w.nocup_cap = len(self.nocup)

    def regrid(self):
        cp = np.zeros((), dtype=CELL_PAR)
        cp["ntags"] = self.ntags
        hi, lo = self.o.cell_dim(self.pp, self.sys)
        cp["rr_max"], cp["rr_min"] = hi, lo
        self.o.grid_from_bbox(cp, self.sys)
        self.set_grid(cp)

    def _arr(self, addr):
        for v in self.bufs.values():
            if v.ctypes.data == addr:
                return v
        raise KeyError(addr)

    @property
    def acc_i(self):
        return self._arr(self.w.acc_i), self._arr(self.w.anga_i)

    @property
    def acc_f(self):
        return self._arr(self.w.acc_f), self._arr(self.w.anga_f)

    def forces(self, phase=PHASE_AVALANCHE, variant=FRICTION_HST) -> int:
        return self.o.lib.orc_forces(_p(self.sys), _p(self.fun), _p(self.cp), _p(self.pp),
                                     C.byref(self.w), int(phase), int(variant))

    def seed_accel(self, phase=PHASE_AVALANCHE, variant=FRICTION_HST) -> int:
        """Start-up force pass into a_i (avalanche_hst.cu:366-384)."""
        st = self.forces(phase, variant)
        self.w.acc_i, self.w.acc_f = self.w.acc_f, self.w.acc_i
        self.w.anga_i, self.w.anga_f = self.w.anga_f, self.w.anga_i
        return st

    def step(self, k=1, phase=PHASE_AVALANCHE, variant=FRICTION_HST, cc0=None, regrid_every=2000) -> int:
        for _ in range(k):
            st = self.o.lib.orc_step(_p(self.sys), _p(self.fun), _p(self.cp), _p(self.pp),
                                     C.byref(self.w), int(phase), int(variant))
            if st:
                return st
            if cc0 is not None:
                if cc0 % regrid_every == 0:
                    self.regrid()
                cc0 += 1
        return 0


class Tangent:
    """The FP64 tangent-linear model (oracle/af3d_tangent.cpp): the oracle over dual numbers."""

    def __init__(self, path: str | None = None):
        if path is None:
            from oracle import build as _b
            path = _b.build_tangent()
        self.lib = C.CDLL(path)
        self.lib.tlm_directions.restype = C.c_int
        self.lib.tlm_run.restype = C.c_int
        self.lib.tlm_run.argtypes = [C.c_void_p] * 4 + [C.c_long, C.c_int, C.c_void_p, C.c_void_p, C.c_long,
                                                        C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        self.ndirs = int(self.lib.tlm_directions())
        self.lib.tlm_set_threads.argtypes = [C.c_int]

    def set_threads(self, n: int) -> None:
        self.lib.tlm_set_threads(int(n))

    def run(self, sys, fun, cp, pp, steps, phase=PHASE_AVALANCHE, variant=FRICTION_HST, dsys=None, dpp=None):
        """Start-up force pass + `steps` steps; returns (J, dJ[ndir], final state).  dsys: array
        of SYSTEM_PAR (one per direction) holding the tangents of the system parameters; dpp:
        array (ndir, n) of PARTICLE holding the tangents of the state."""
        sys = np.ascontiguousarray(np.array(sys, dtype=SYSTEM_PAR))
        fun = np.ascontiguousarray(np.array(fun, dtype=FUNNEL))
        cp = np.ascontiguousarray(np.array(cp, dtype=CELL_PAR))
        pp = np.ascontiguousarray(pp, dtype=PARTICLE)
        n = len(pp)
        ndir = len(dsys) if dsys is not None else (len(dpp) if dpp is not None else 0)
        if ndir > self.ndirs:
            raise ValueError("at most %d directions per run" % self.ndirs)
        if dsys is not None:
            dsys = np.ascontiguousarray(dsys, dtype=SYSTEM_PAR)
            assert len(dsys) == ndir
        if dpp is not None:
            dpp = np.ascontiguousarray(dpp, dtype=PARTICLE)
            assert dpp.shape == (ndir, n)
        J = C.c_double()
        dJ = np.zeros(max(ndir, 1))
        out = np.zeros(n, dtype=PARTICLE)
        st = self.lib.tlm_run(_p(sys), _p(fun), _p(cp), _p(pp) if n else None, n, ndir,
                              _p(dsys) if dsys is not None else None, _p(dpp) if dpp is not None else None,
                              int(steps), int(phase), int(variant), C.byref(J), _p(dJ), _p(out) if n else None)
        if st != 0:
            raise RuntimeError("tlm_run failed with status %d" % st)
        return J.value, dJ[:ndir].copy(), out


def state_tangent(pp: np.ndarray, sys, dr=None, dv=None, dw=None, dphi=None) -> np.ndarray:
    """A PARTICLE-layout tangent of the state pp: position, velocity and angular-velocity
    tangents (n, 3), and an orientation tangent dR = K(dphi) R (K the skew matrix of dphi, R's
    rows Rmatx, Rmaty, Rmatz); the sphere centres follow r and R (init_Verlet.cu:130-142 is
    linear in both) and the slope-frame copies rrot, rrot_s follow r and the sphere centres
    (rotate_vectors.cu:28-46, linear; the wall routines of the start-up pass read them)."""
    n = len(pp)
    t = np.zeros(n, dtype=PARTICLE)
    if dr is not None:
        t["rr"] = dr
    if dv is not None:
        t["vv"] = dv
    if dw is not None:
        t["ww"] = dw
    if dphi is not None:
        R = np.stack([pp["Rmatx"], pp["Rmaty"], pp["Rmatz"]], 1)
        k = np.asarray(dphi, dtype=np.float64)
        K = np.zeros((n, 3, 3))
        K[:, 0, 1], K[:, 0, 2], K[:, 1, 2] = -k[:, 2], k[:, 1], -k[:, 0]
        K[:, 1, 0], K[:, 2, 0], K[:, 2, 1] = k[:, 2], -k[:, 1], k[:, 0]
        dR = K @ R
        t["Rmatx"], t["Rmaty"], t["Rmatz"] = dR[:, 0], dR[:, 1], dR[:, 2]
    t["radius"] = pp["radius"]
    sphere_centres(t)
    t["radius"] = 0.0
    rotate_slope(t, sys)
    return t
