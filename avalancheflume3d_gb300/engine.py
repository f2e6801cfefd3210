"""Host-side mirror of the reference's step interface over the C ABI (include/af3d.h).

``Engine`` holds one device-resident context.  Its methods are named after the reference's
routines and keep their argument meaning (system_par / Funnel / particle / cell_par as numpy
structured scalars and arrays with the reference's binary layout); the step loop of
avalanche_hst.cu:668-710 reads::

    eng.init_verlet(); eng.advance_time(); eng.rotate_vectors(); eng.clear_forces()
    eng.cell_build()
    for nw in range(3): eng.force_hop(nw)
    eng.force_funnel(); eng.force_fcorners(); eng.force_walls()
    eng.force_part(0)            # all sixteen sph_id passes in one call
    eng.force_flume(); eng.get_accel(); eng.finish_verlet(); eng.swap_accel()

or, fused and graph-captured, ``eng.step(k)``.  Errors raise :class:`EngineError` with the
AF3D_ERR_* code; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (CELL_PAR, FP_EXACT, FRICTION_HST, FUNNEL, INPUTS, OBJ_CENTROID, OBJ_RUNOUT, PARTICLE,
                   PHASE_AVALANCHE, RNG,
                   SYSTEM_PAR, EngineError, Vec3, check, lib, ptr)


def _vec3(n: int) -> np.ndarray:
    return np.zeros((n, 3), dtype=np.float64)


class Engine:
    """One simulation context on the current CUDA device.

    ``sys``/``fun`` as structured scalars give the reference's single flume; as 1-d arrays of
    length F they give a batched ensemble of F independent flumes (clump ids flume after flume,
    shared dt and clock; see ``af3d_create_ensemble``)."""

    def __init__(self, sys: np.ndarray, fun: np.ndarray, ntags: int = 9, phase: int = PHASE_AVALANCHE,
                 friction: int = FRICTION_HST, stream: int | None = None, fp_mode: int = FP_EXACT):
        L = lib()
        self._L = L
        sys_a = np.array(sys, dtype=SYSTEM_PAR)
        fun_a = np.array(fun, dtype=FUNNEL)
        self.ensemble = sys_a.ndim == 1
        sys_a = np.ascontiguousarray(sys_a.reshape(-1)).copy()
        fun_a = np.ascontiguousarray(fun_a.reshape(-1)).copy()
        if len(fun_a) != len(sys_a):
            raise ValueError("one Funnel per flume")
        self.nflumes = len(sys_a)
        self.flume_sizes = [int(s["npart"]) for s in sys_a]
        self.first_id = np.concatenate([[0], np.cumsum(self.flume_sizes)]).astype(np.int64)
        self.n = int(self.first_id[-1])
        self.sys = sys_a if self.ensemble else sys_a.reshape(()).copy()
        self.fun = fun_a if self.ensemble else fun_a.reshape(()).copy()
        h = C.c_void_p()
        check(L.af3d_create_ensemble(self.nflumes, ptr(sys_a), ptr(fun_a), int(ntags), int(phase),
                                     C.byref(h)), "af3d_create_ensemble")
        self._h = h
        if friction != FRICTION_HST:
            self.set_friction(friction)
        if stream:
            check(L.af3d_set_stream(h, C.c_void_p(stream)), "af3d_set_stream")
        if fp_mode != FP_EXACT:
            self.set_fp_mode(fp_mode)

    # ---- lifetime ----
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.af3d_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _call(self, name: str, *args) -> None:
        check(getattr(self._L, name)(self._h, *args), name)

    # ---- state in/out ----
    def import_particles(self, pp: np.ndarray, acc: np.ndarray | None = None,
                         anga: np.ndarray | None = None) -> None:
        pp = np.ascontiguousarray(pp, dtype=PARTICLE)
        assert pp.shape == (self.n,)
        a = None if acc is None else np.ascontiguousarray(acc, dtype=np.float64)
        al = None if anga is None else np.ascontiguousarray(anga, dtype=np.float64)
        self._call("af3d_import_particles", ptr(pp), ptr(a), ptr(al))

    def export_particles(self, with_accel: bool = True):
        pp = np.zeros(self.n, dtype=PARTICLE)
        a = _vec3(self.n) if with_accel else None
        al = _vec3(self.n) if with_accel else None
        self._call("af3d_export_particles", ptr(pp), ptr(a), ptr(al))
        return (pp, a, al) if with_accel else pp

    def step_host(self, pp: np.ndarray, acc: np.ndarray | None = None, anga: np.ndarray | None = None,
                  out: np.ndarray | None = None, acc_out: np.ndarray | None = None,
                  anga_out: np.ndarray | None = None) -> None:
        """af3d_step_host: import pp (and accelerations), one step, export into out (default: pp
        itself) and acc_out/anga_out, with the export overlapping the force pass."""
        pp = np.ascontiguousarray(pp, dtype=PARTICLE)
        assert pp.shape == (self.n,)
        out = pp if out is None else out
        assert out.dtype == PARTICLE and out.shape == (self.n,) and out.flags.c_contiguous
        for a in (acc, anga, acc_out, anga_out):
            assert a is None or (a.dtype == np.float64 and a.shape == (self.n, 3) and a.flags.c_contiguous)
        self._call("af3d_step_host", ptr(pp), ptr(acc), ptr(anga), ptr(out), ptr(acc_out), ptr(anga_out))

    def prepare_steps(self, k: int) -> None:
        """af3d_prepare_steps: capture the graphs the next step(k) replays, running nothing."""
        self._call("af3d_prepare_steps", int(k))

    def set_resort_every(self, steps: int) -> None:
        """af3d_set_resort_every: steps between permutations of the planes into cell order."""
        self._call("af3d_set_resort_every", int(steps))

    RESORT_CHOICES = (16, 32, 64, 128, 256)

    def autotune(self, steps_per_trial: int = 256, timings: dict | None = None) -> int:
        """af3d_autotune: time each permutation interval on real steps of the run, keep the
        fastest, return it (the trajectory does not depend on it); `timings` receives each
        interval's ms per step."""
        r = C.c_long()
        ms = np.zeros(len(self.RESORT_CHOICES))
        self._call("af3d_autotune", int(steps_per_trial), C.byref(r), ptr(ms))
        if timings is not None:
            timings.update(zip(self.RESORT_CHOICES, ms.tolist()))
        return r.value

    FORCE_BLOCKS = (128, 96, 64, 192)

    def set_force_block(self, block: int) -> None:
        """af3d_set_force_block: threads per block of the fused force kernel (64, 96, 128 or 192)."""
        self._call("af3d_set_force_block", int(block))

    def force_block(self) -> int:
        b = C.c_int()
        self._call("af3d_get_force_block", C.byref(b))
        return b.value

    def autotune_shapes(self, steps_per_trial: int = 256, timings: dict | None = None) -> tuple[int, int]:
        """af3d_autotune_shapes: the permutation interval, then the force kernel's block, each the
        fastest on real steps of the run; returns (interval, block).  `timings` receives
        {"interval": {every: ms}, "block": {block: ms}}."""
        r, b = C.c_long(), C.c_int()
        mi, mb = np.zeros(len(self.RESORT_CHOICES)), np.zeros(len(self.FORCE_BLOCKS))
        self._call("af3d_autotune_shapes", int(steps_per_trial), C.byref(r), C.byref(b), ptr(mi), ptr(mb))
        if timings is not None:
            timings["interval"] = dict(zip(self.RESORT_CHOICES, mi.tolist()))
            timings["block"] = dict(zip(self.FORCE_BLOCKS, mb.tolist()))
        return r.value, b.value

    def save_checkpoint(self, path: str) -> None:
        """af3d_save_checkpoint: the whole context state, losslessly, to `path`."""
        self._call("af3d_save_checkpoint", str(path).encode())

    def load_checkpoint(self, path: str) -> None:
        """af3d_load_checkpoint: a checkpoint of a context of the same shape."""
        self._call("af3d_load_checkpoint", str(path).encode())
        self.sys = self.get_system() if not self.ensemble else self.sys

    def set_system(self, sys: np.ndarray) -> None:
        """system_par of flume 0 (the only flume of a plain context)."""
        s = np.array(sys, dtype=SYSTEM_PAR).reshape(1).copy()
        self._call("af3d_set_system", ptr(s))
        if not self.ensemble:
            self.sys = s.reshape(()).copy()

    def get_system(self) -> np.ndarray:
        s = np.zeros(1, dtype=SYSTEM_PAR)
        self._call("af3d_get_system", ptr(s))
        s = s.reshape(()).copy()
        if not self.ensemble:
            self.sys = s
        return s

    def set_grid(self, cell: np.ndarray) -> None:
        c = np.array(cell, dtype=CELL_PAR).reshape(1).copy()
        self._call("af3d_set_grid", ptr(c))

    def get_grid(self) -> np.ndarray:
        c = np.zeros(1, dtype=CELL_PAR)
        self._call("af3d_get_grid", ptr(c))
        return c.reshape(()).copy()

    # ---- per flume of an ensemble ----
    def flume_slice(self, f: int) -> slice:
        """Clump ids of flume f."""
        return slice(int(self.first_id[f]), int(self.first_id[f + 1]))

    def set_flume_system(self, f: int, sys: np.ndarray, fun: np.ndarray | None = None) -> None:
        s = np.array(sys, dtype=SYSTEM_PAR).reshape(1).copy()
        u = None if fun is None else np.array(fun, dtype=FUNNEL).reshape(1).copy()
        self._call("af3d_set_flume_system", int(f), ptr(s), ptr(u))

    def get_flume_system(self, f: int) -> np.ndarray:
        s = np.zeros(1, dtype=SYSTEM_PAR)
        self._call("af3d_get_flume_system", int(f), ptr(s))
        return s.reshape(()).copy()

    def set_flume_grid(self, f: int, cell: np.ndarray) -> None:
        c = np.array(cell, dtype=CELL_PAR).reshape(1).copy()
        self._call("af3d_set_flume_grid", int(f), ptr(c))

    def get_flume_grid(self, f: int) -> np.ndarray:
        c = np.zeros(1, dtype=CELL_PAR)
        self._call("af3d_get_flume_grid", int(f), ptr(c))
        return c.reshape(()).copy()

    def flume_count(self) -> int:
        return int(self._L.af3d_flume_count(self._h))

    def set_fp_mode(self, mode: int) -> None:
        """FP_EXACT (bit-identical to the reference) or FP_FAST (contracted FP64) for step/forces."""
        self._call("af3d_set_fp_mode", int(mode))

    def set_friction(self, variant: int) -> None:
        self._call("af3d_set_friction", int(variant))

    def set_phase(self, phase: int) -> None:
        self._call("af3d_set_phase", int(phase))

    def regrid(self) -> None:
        self._call("af3d_regrid")

    def open_door(self) -> None:
        self._call("af3d_open_door")

    # ---- one call per reference routine ----
    def init_verlet(self): self._call("af3d_init_verlet")
    def advance_time(self): self._call("af3d_advance_time")
    def rotate_vectors(self): self._call("af3d_rotate_vectors")
    def clear_forces(self): self._call("af3d_clear_forces")
    def cell_build(self): self._call("af3d_cell_build")
    def force_hop(self, nw: int): self._call("af3d_force_hop", int(nw))
    def force_funnel(self): self._call("af3d_force_funnel")
    def force_fcorners(self): self._call("af3d_force_fcorners")
    def force_walls(self): self._call("af3d_force_walls")
    def force_part(self, sph_id: int = 0): self._call("af3d_force_part", int(sph_id))
    def force_flume(self): self._call("af3d_force_flume")
    def get_accel(self): self._call("af3d_get_accel")
    def finish_verlet(self): self._call("af3d_finish_verlet")
    def swap_accel(self): self._call("af3d_swap_accel")

    # ---- fused paths ----
    def forces(self) -> None:
        """clear_forces + cells + every force routine of the phase + get_accel (into a_f)."""
        self._call("af3d_forces")

    def step(self, k: int = 1) -> None:
        """k fused steps of the current phase (CUDA-graph replay, re-grid every 2000 steps)."""
        self._call("af3d_step", int(k))

    # ---- adjoint ----
    def adjoint(self, steps: int, ckpt_every: int = 500, gradients: bool = True, runout: float | None = None) -> dict:
        """Start-up force pass + `steps` exact steps from the imported state, J at the end and
        (gradients=True) dJ/d(parameters, initial state) from the hand-written adjoint
        (af3d_adjoint).  J is the mass-weighted mean downslope position (the deposit centroid),
        or with ``runout`` = l > 0 [cm] the runout l ln(sum m exp(x / l) / sum m), a soft maximum
        of the downslope positions.  Leaves the context at the final state.

        For an ensemble, ``J`` is an array over flumes and every ``params`` entry an array of
        each flume's own derivative; the per-clump gradients are those of the clump's flume."""
        if runout is None:
            self._call("af3d_set_objective", OBJ_CENTROID, 0.0)
        else:
            self._call("af3d_set_objective", OBJ_RUNOUT, float(runout))
        names = ("kappa_pp", "gamma_pp", "mu_pp", "kappa_pw", "gamma_pw", "mu_pw")
        J = np.zeros(self.nflumes)
        out = {}
        if gradients:
            pg = np.zeros((self.nflumes, 6))
            dr, dv, dw = _vec3(self.n), _vec3(self.n), _vec3(self.n)
            dR = np.zeros((self.n, 9))
            self._call("af3d_adjoint", int(steps), int(ckpt_every), ptr(J), ptr(pg), ptr(dr), ptr(dR), ptr(dv),
                       ptr(dw))
            params = {k: (pg[:, i].copy() if self.ensemble else float(pg[0, i])) for i, k in enumerate(names)}
            out.update(params=params, r0=dr, v0=dv, w0=dw, R0=dR.reshape(-1, 3, 3))
        else:
            self._call("af3d_adjoint", int(steps), int(ckpt_every), ptr(J), None, None, None, None, None)
        out["J"] = J if self.ensemble else float(J[0])
        return out

    # ---- diagnostics (indexed by clump id) ----
    def status(self) -> int:
        f = C.c_int()
        self._call("af3d_get_status", C.byref(f))
        return f.value

    def get_forces(self):
        F, T = _vec3(self.n), _vec3(self.n)
        self._call("af3d_get_forces", ptr(F), ptr(T))
        return F, T

    def get_accels(self):
        a, al = _vec3(self.n), _vec3(self.n)
        self._call("af3d_get_accels", ptr(a), ptr(al))
        return a, al

    def get_cells(self):
        """(cell of every clump or -1, (cell, id)-sorted ids of the binned clumps)."""
        cell = np.zeros(self.n, dtype=np.int64)
        ids = np.zeros(self.n, dtype=np.int64)
        nb = C.c_long()
        self._call("af3d_get_cells", ptr(cell), ptr(ids), C.byref(nb))
        return cell, ids[:nb.value].copy()

    def contact_pairs(self, active: bool = False) -> np.ndarray:
        cap = max(1024, 64 * self.n)
        while True:
            out = np.zeros((cap, 3), dtype=np.int64)
            cnt = C.c_long()
            self._call("af3d_contact_pairs", ptr(out), cap, C.byref(cnt), int(bool(active)))
            if cnt.value <= cap:
                return out[:cnt.value].copy()
            cap = cnt.value

    def contact_count(self) -> int:
        c = C.c_long()
        self._call("af3d_contact_count", C.byref(c))
        return c.value

    def list_overflows(self) -> int:
        """Clumps whose item lists overflowed in the fused force passes since the last call
        (their contacts ran by the per-clump cell walk)."""
        c = C.c_long()
        self._call("af3d_list_overflows", C.byref(c))
        return c.value


# ---- host I/O and generators (no GPU) ----

def load_datainput(path: str) -> np.ndarray:
    v = np.zeros(1, dtype=INPUTS)
    check(lib().af3d_load_datainput(path.encode(), ptr(v)), "af3d_load_datainput")
    return v.reshape(()).copy()


def derive_system(inputs: np.ndarray):
    s = np.zeros(1, dtype=SYSTEM_PAR)
    f = np.zeros(1, dtype=FUNNEL)
    v = np.array(inputs, dtype=INPUTS).reshape(1)
    check(lib().af3d_derive_system(ptr(v), ptr(s), ptr(f)), "af3d_derive_system")
    return s.reshape(()).copy(), f.reshape(()).copy()


def error_check(sys: np.ndarray) -> tuple[int, str]:
    buf = C.create_string_buffer(512)
    s = np.array(sys, dtype=SYSTEM_PAR).reshape(1)
    n = lib().af3d_error_check(ptr(s), buf, 512)
    return n, buf.value.decode()


def write_last_config(path: str, pp: np.ndarray, aval_start: int, time: float, cc: int, jj: int):
    pp = np.ascontiguousarray(pp, dtype=PARTICLE)
    check(lib().af3d_write_last_config(path.encode(), int(aval_start), float(time), int(cc), int(jj),
                                       ptr(pp), len(pp)), "af3d_write_last_config")


def read_last_config(path: str, pp: np.ndarray):
    """Fill rr, R, vv, ww (and the sphere centres) of ``pp`` in place; returns the header."""
    a, cc, jj = C.c_int(), C.c_long(), C.c_long()
    t = C.c_double()
    check(lib().af3d_read_last_config(path.encode(), C.byref(a), C.byref(t), C.byref(cc), C.byref(jj),
                                      ptr(pp), len(pp)), "af3d_read_last_config")
    return a.value, t.value, cc.value, jj.value


def append_snapshot(pp: np.ndarray, sys: np.ndarray, phase: int, xyz: str | None = None, vel: str | None = None,
                    vmean: str | None = None, xcm: str | None = None) -> None:
    """One frame of the reference's snapshot files (.xyz spheres, velocity field, mean-velocity
    and centre-of-mass CSV lines), appended to the given paths (None: skipped)."""
    pp = np.ascontiguousarray(pp, dtype=PARTICLE)
    s = np.array(sys, dtype=SYSTEM_PAR).reshape(1)
    enc = lambda x: None if x is None else str(x).encode()
    check(lib().af3d_append_snapshot(enc(xyz), enc(vel), enc(vmean), enc(xcm), ptr(pp), len(pp), ptr(s), int(phase)),
          "af3d_append_snapshot")


class Rannew64:
    """The reference's rannew64 generator (rannew64.cu:55) with explicit state."""

    def __init__(self, idum: int):
        self._s = RNG()
        lib().af3d_rng_seed(C.byref(self._s), int(idum))

    def __call__(self) -> float:
        return lib().af3d_rng_next(C.byref(self._s))

    @property
    def ref(self):
        return C.byref(self._s)

    def clone(self) -> "Rannew64":
        """An independent generator in this one's state."""
        g = Rannew64.__new__(Rannew64)
        g._s = RNG.from_buffer_copy(self._s)
        return g

    def assign(self, other: "Rannew64") -> None:
        """Take over `other`'s state."""
        C.memmove(C.addressof(self._s), C.addressof(other._s), C.sizeof(RNG))


def generate_particles(sys: np.ndarray) -> np.ndarray:
    n = int(sys["npart"])
    pp = np.zeros(n, dtype=PARTICLE)
    s = np.array(sys, dtype=SYSTEM_PAR).reshape(1)
    lib().af3d_generate_particles(ptr(pp), ptr(s))
    return pp


def calculate_particle_parameters(pp: np.ndarray) -> None:
    lib().af3d_calculate_particle_parameters(ptr(pp), len(pp))


def place_particles(sys: np.ndarray, pp: np.ndarray) -> None:
    s = np.array(sys, dtype=SYSTEM_PAR).reshape(1)
    check(lib().af3d_place_particles(ptr(s), ptr(pp)), "af3d_place_particles")


def set_initial_velocity(sys: np.ndarray, pp: np.ndarray) -> None:
    s = np.array(sys, dtype=SYSTEM_PAR).reshape(1)
    lib().af3d_set_initial_velocity(ptr(s), ptr(pp))


def sphere_centres(pp: np.ndarray) -> None:
    lib().af3d_sphere_centres(ptr(pp), len(pp))


def lattice_block(pp: np.ndarray, lo, hi, pitch: float, rng: Rannew64, max_tries: int = 64) -> int:
    return int(lib().af3d_lattice_block(ptr(pp), len(pp), Vec3(*lo), Vec3(*hi), float(pitch), rng.ref,
                                        int(max_tries)))


def lattice_pile(pp: np.ndarray, lo, hi, pitch: float, overlap: float, rng: Rannew64,
                 max_tries: int = 64) -> int:
    return int(lib().af3d_lattice_pile(ptr(pp), len(pp), Vec3(*lo), Vec3(*hi), float(pitch),
                                       float(overlap), rng.ref, int(max_tries)))


__all__ = ["Engine", "EngineError", "load_datainput", "derive_system", "error_check",
           "write_last_config", "read_last_config", "Rannew64", "generate_particles",
           "calculate_particle_parameters", "place_particles", "set_initial_velocity",
           "sphere_centres", "lattice_block", "lattice_pile"]
