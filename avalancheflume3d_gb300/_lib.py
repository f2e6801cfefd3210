"""ctypes binding of ``libaf3d.so`` (the C ABI of include/af3d.h).

The library is built in-tree by :mod:`avalancheflume3d_gb300.build`.  Loading fails loudly when
it is missing: there is no CPU fallback for the engine.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libaf3d.so")

VEC3 = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8")])

# Layouts equal to the reference's structs (cabecera.hu:34-112).
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
INPUTS = np.dtype([("npart", "<i8")] + [(f, "<f8") for f in (
    "width", "hopper_height", "rmin", "rmax", "v0", "dt", "eps_pw", "mu_pw", "eps_pp", "mu_pp",
    "t_coll", "Lflume", "tilt_deg")] + [("ntags", "<i8"), ("print_flag", "<i4"), ("_pad", "<i4")])
assert SYSTEM_PAR.itemsize == 256 and PARTICLE.itemsize == 408 and CELL_PAR.itemsize == 168


class Vec3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class RNG(C.Structure):
    _fields_ = [("seed", C.c_uint64 * 250), ("uy", C.c_uint64), ("np", C.c_int), ("nq", C.c_int),
                ("init", C.c_int)]


OK = 0
ERRORS = {1: "ARG", 2: "CUDA", 3: "NOMEM", 4: "GRID_ESCAPE", 5: "NEGATIVE_CELL",
          6: "CELL_CAPACITY", 7: "NAN", 8: "IO", 9: "INPUT"}
FRICTION_HST, FRICTION_DEV = 0, 1
PHASE_FILL, PHASE_AVALANCHE = 0, 1
FP_EXACT, FP_FAST = 0, 1
OBJ_CENTROID, OBJ_RUNOUT = 0, 1

# (name, argtypes, restype) of every exported entry point of include/af3d.h.
_P = C.c_void_p
SIGNATURES = [
    ("af3d_create", [_P, _P, C.c_long, C.c_int, _P], C.c_int),
    ("af3d_destroy", [_P], C.c_int),
    ("af3d_set_stream", [_P, _P], C.c_int),
    ("af3d_set_friction", [_P, C.c_int], C.c_int),
    ("af3d_set_fp_mode", [_P, C.c_int], C.c_int),
    ("af3d_last_error", [], C.c_char_p),
    ("af3d_abi_version", [], C.c_int),
    ("af3d_import_particles", [_P, _P, _P, _P], C.c_int),
    ("af3d_export_particles", [_P, _P, _P, _P], C.c_int),
    ("af3d_step_host", [_P, _P, _P, _P, _P, _P, _P], C.c_int),
    ("af3d_save_checkpoint", [_P, C.c_char_p], C.c_int),
    ("af3d_set_resort_every", [_P, C.c_long], C.c_int),
    ("af3d_prepare_steps", [_P, C.c_long], C.c_int),
    ("af3d_autotune", [_P, C.c_long, _P, _P], C.c_int),
    ("af3d_load_checkpoint", [_P, C.c_char_p], C.c_int),
    ("af3d_set_system", [_P, _P], C.c_int),
    ("af3d_get_system", [_P, _P], C.c_int),
    ("af3d_set_grid", [_P, _P], C.c_int),
    ("af3d_get_grid", [_P, _P], C.c_int),
    ("af3d_create_ensemble", [C.c_int, _P, _P, C.c_long, C.c_int, _P], C.c_int),
    ("af3d_flume_count", [_P], C.c_int),
    ("af3d_set_flume_system", [_P, C.c_int, _P, _P], C.c_int),
    ("af3d_get_flume_system", [_P, C.c_int, _P], C.c_int),
    ("af3d_set_flume_grid", [_P, C.c_int, _P], C.c_int),
    ("af3d_get_flume_grid", [_P, C.c_int, _P], C.c_int),
    ("af3d_set_phase", [_P, C.c_int], C.c_int),
    ("af3d_regrid", [_P], C.c_int),
    ("af3d_open_door", [_P], C.c_int),
    ("af3d_init_verlet", [_P], C.c_int),
    ("af3d_advance_time", [_P], C.c_int),
    ("af3d_rotate_vectors", [_P], C.c_int),
    ("af3d_clear_forces", [_P], C.c_int),
    ("af3d_cell_build", [_P], C.c_int),
    ("af3d_force_hop", [_P, C.c_int], C.c_int),
    ("af3d_force_funnel", [_P], C.c_int),
    ("af3d_force_fcorners", [_P], C.c_int),
    ("af3d_force_walls", [_P], C.c_int),
    ("af3d_force_part", [_P, C.c_int], C.c_int),
    ("af3d_force_flume", [_P], C.c_int),
    ("af3d_get_accel", [_P], C.c_int),
    ("af3d_finish_verlet", [_P], C.c_int),
    ("af3d_swap_accel", [_P], C.c_int),
    ("af3d_forces", [_P], C.c_int),
    ("af3d_step", [_P, C.c_long], C.c_int),
    ("af3d_get_status", [_P, _P], C.c_int),
    ("af3d_adjoint", [_P, C.c_long, C.c_long, _P, _P, _P, _P, _P, _P], C.c_int),
    ("af3d_set_objective", [_P, C.c_int, C.c_double], C.c_int),
    ("af3d_set_force_block", [_P, C.c_int], C.c_int),
    ("af3d_get_force_block", [_P, _P], C.c_int),
    ("af3d_autotune_shapes", [_P, C.c_long, _P, _P, _P, _P], C.c_int),
    ("af3d_step_profile", [_P, C.c_long, _P], C.c_int),
    ("af3d_kernel_launches", [_P, _P], C.c_int),
    ("af3d_fp64_peak", [_P], C.c_int),
    ("af3d_check_fp64_bits", [_P, C.c_long, _P], C.c_int),
    ("af3d_get_forces", [_P, _P, _P], C.c_int),
    ("af3d_get_accels", [_P, _P, _P], C.c_int),
    ("af3d_get_cells", [_P, _P, _P, _P], C.c_int),
    ("af3d_contact_pairs", [_P, _P, C.c_long, _P, C.c_int], C.c_int),
    ("af3d_contact_count", [_P, _P], C.c_int),
    ("af3d_list_overflows", [_P, _P], C.c_int),
    ("af3d_contact_pairs_noalloc", [_P, _P, C.c_long, _P, C.c_int], C.c_int),
    ("af3d_load_datainput", [C.c_char_p, _P], C.c_int),
    ("af3d_read_datainput", [_P, _P], C.c_int),
    ("af3d_derive_system", [_P, _P, _P], C.c_int),
    ("af3d_error_check", [_P, C.c_char_p, C.c_size_t], C.c_int),
    ("af3d_write_last_config", [C.c_char_p, C.c_int, C.c_double, C.c_long, C.c_long, _P, C.c_long], C.c_int),
    ("af3d_read_last_config", [C.c_char_p, _P, _P, _P, _P, _P, C.c_long], C.c_int),
    ("af3d_append_snapshot", [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, _P, C.c_long, _P, C.c_int],
     C.c_int),
    ("af3d_rng_seed", [_P, C.c_long], None),
    ("af3d_rng_next", [_P], C.c_double),
    ("af3d_generate_particles", [_P, _P], None),
    ("af3d_calculate_particle_parameters", [_P, C.c_long], None),
    ("af3d_place_particles", [_P, _P], C.c_int),
    ("af3d_set_initial_velocity", [_P, _P], None),
    ("af3d_sphere_centres", [_P, C.c_long], None),
    ("af3d_lattice_block", [_P, C.c_long, Vec3, Vec3, C.c_double, _P, C.c_int], C.c_long),
    ("af3d_lattice_pile", [_P, C.c_long, Vec3, Vec3, C.c_double, C.c_double, _P, C.c_int], C.c_long),
]

_lib = None


class EngineError(RuntimeError):
    def __init__(self, code: int, where: str):
        self.code = code
        msg = ""
        if _lib is not None:
            msg = (_lib.af3d_last_error() or b"").decode(errors="replace")
        super().__init__("%s failed: AF3D_ERR_%s (%d) %s" % (where, ERRORS.get(code, "?"), code, msg))


def lib() -> C.CDLL:
    """The loaded engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libaf3d.so is missing: build it with `python -c \"import __graft_entry__ as g; "
                              "g.build()\"` (no CPU fallback exists)")
        L = C.CDLL(LIB_PATH)
        for name, args, res in SIGNATURES:
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def check(code: int, where: str) -> None:
    if code != OK:
        raise EngineError(code, where)


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)
