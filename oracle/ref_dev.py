"""The reference's OWN device kernels on the GPU -- TEST AND MEASUREMENT INFRASTRUCTURE ONLY.

``oracle/build.py`` compiles the reference's ``*_dev`` kernels from its unmodified sources into
``oracle/_ref/dev/<file>.cubin`` (sm_103a, the Makefile's ``-O2``).  This module loads those
modules through the CUDA driver API (ctypes on ``libcuda.so.1``, in the context PyTorch made
current) and drives them in the reference's own device step sequence:

* :meth:`RefDeviceRun.seed_accel` -- the start-up force pass of ``avalanche_dev.cu:335-360``
  (clear_forces, clear_cell, clear_ocup, cell_locate, force_part x16, force_hop x3, get_accel
  into a_i)
* :meth:`RefDeviceRun.step` -- ``avalanche_dev.cu:636-693`` per step: init_Verlet, time += dt,
  rotate_vectors, clear_forces, clear_cell, clear_ocup, cell_locate, force_hop x3,
  force_funnel, force_fcorners, force_walls, force_part x16, force_flume, get_accel,
  finish_Verlet, then the a_i/a_f swap; 256 threads per block, grids as ``avalanche_dev.cu:161-162,
  329-330``.

The engine's product path never imports it: it serves the GPU parity test of the engine
against the reference's kernels and the reference-GPU line of the benchmark.

``cell_locate_dev`` (``cells.cu:150-202``) checks no bounds: a clump outside the grid, or a cell
holding more than ``ntags`` clumps, would write outside ``cell_vec``.  :func:`grid_margin` and
:func:`max_occupancy` measure both on the host.  :class:`RefDeviceRun` refuses a state whose
clumps are not at least ``min_margin`` cells inside the grid or whose fullest cell holds more than
half of ``ntags``, and :meth:`RefDeviceRun.step_checked` checks the positions every next step's
predictor will produce before launching it.  A timed run repeats, from a snapshot, a sequence a
checked run has just completed (the same kernels on the same state: only the summation order of
the binning race differs, by rounding)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from oracle.pyoracle import CELL_PAR, FUNNEL, PARTICLE, SYSTEM_PAR

DEV_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "dev")
NTHREAD = 256   # avalanche_dev.cu:161

# kernel -> (module, argument kinds): P device pointer, s system_par, c cell_par, f Funnel,
# b char, i int (the reference's prototypes, cabecera.hu:115-157)
KERNELS = {
    "init_Verlet_dev": ("init_Verlet", "PPsP"),
    "rotate_vectors_dev": ("rotate_vectors", "Ps"),
    "clear_forces_dev": ("clear_forces", "sPP"),
    "clear_cell_dev": ("cells", "cP"),
    "clear_ocup_dev": ("cells", "cP"),
    "cell_locate_dev": ("cells", "csPPP"),
    "force_hop_dev": ("force_hop", "PPsPb"),
    "force_funnel_dev": ("force_funnel", "PPsPf"),
    "force_fcorners_dev": ("force_funnel", "PPsfP"),
    "force_walls_dev": ("force_walls", "PPsP"),
    "force_part_dev": ("force_part", "PPPPPsci"),
    "force_flume_dev": ("force_flume", "PPsP"),
    "get_accel_dev": ("get_accel", "PPPPsP"),
    "finish_Verlet_dev": ("finish_Verlet", "PPPPsP"),
}


def available() -> bool:
    return all(os.path.exists(os.path.join(DEV_DIR, m + ".cubin")) for m, _ in KERNELS.values())


def cell_coords(pp: np.ndarray, cp) -> np.ndarray:
    """cell_locate_dev's (i, j, k) per clump as reals (cs_inv (r - rr_min), before truncation)."""
    return (pp["rr"] - np.asarray(cp["rr_min"])) * np.asarray(cp["cs_inv"])


def _active(pp: np.ndarray, sys) -> np.ndarray:
    # the removal rule of cells.cu:171 (time > 0 and x > side.x): those clumps are not binned
    return ~((float(sys["time"]) > 0.0) & (pp["rr"][:, 0] > float(sys["side"][0])))


def grid_margin(pp: np.ndarray, cp, sys) -> float:
    """Smallest distance, in cells, of a binned clump from the grid's faces (negative: outside)."""
    q = cell_coords(pp, cp)[_active(pp, sys)]
    if len(q) == 0:
        return float("inf")
    nc = np.asarray(cp["ncell"], dtype=np.float64)
    return float(min(q.min(), (nc - q).min()))


def max_occupancy(pp: np.ndarray, cp, sys) -> int:
    """Clumps in the fullest cell, with cell_locate_dev's index arithmetic."""
    q = cell_coords(pp, cp)[_active(pp, sys)]
    if len(q) == 0:
        return 0
    nc = np.asarray(cp["ncell"], dtype=np.int64)
    ijk = q.astype(np.int64)
    ijk = np.where(ijk == nc, ijk - 1, ijk)
    idx = ijk[:, 0] + nc[0] * (ijk[:, 1] + nc[1] * ijk[:, 2])
    return int(np.bincount(idx).max())


class _Driver:
    """The CUDA driver API entry points used here, in the calling thread's current context."""

    def __init__(self):
        import torch
        torch.zeros(1, device="cuda")   # the primary context, current in this thread
        self.cu = C.CDLL("libcuda.so.1")
        cu = self.cu
        for name in ("cuModuleLoad", "cuModuleGetFunctionCount", "cuModuleEnumerateFunctions", "cuFuncGetName",
                     "cuLaunchKernel", "cuModuleUnload", "cuGetErrorString", "cuCtxGetCurrent"):
            if not hasattr(cu, name):
                raise RuntimeError("CUDA driver lacks " + name)
        cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                      C.c_uint, C.c_void_p, C.c_void_p, C.c_void_p]
        ctx = C.c_void_p()
        self.check(cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")

    def check(self, r: int, what: str) -> None:
        if r != 0:
            s = C.c_char_p()
            self.cu.cuGetErrorString(r, C.byref(s))
            raise RuntimeError("%s: CUDA driver error %d (%s)" % (what, r, s.value.decode() if s.value else "?"))

    def load(self, path: str) -> tuple[C.c_void_p, dict[str, C.c_void_p]]:
        mod = C.c_void_p()
        self.check(self.cu.cuModuleLoad(C.byref(mod), path.encode()), "cuModuleLoad " + path)
        n = C.c_uint()
        self.check(self.cu.cuModuleGetFunctionCount(C.byref(n), mod), "cuModuleGetFunctionCount")
        fns = (C.c_void_p * n.value)()
        self.check(self.cu.cuModuleEnumerateFunctions(fns, n, mod), "cuModuleEnumerateFunctions")
        out = {}
        for f in fns:
            name = C.c_char_p()
            self.check(self.cu.cuFuncGetName(C.byref(name), C.c_void_p(f)), "cuFuncGetName")
            out[name.value.decode()] = C.c_void_p(f)
        return mod, out


def _find(funcs: dict[str, C.c_void_p], kernel: str) -> C.c_void_p:
    # the Itanium-mangled name of a free function starts with _Z<length><name>
    pre = "_Z%d%s" % (len(kernel), kernel)
    hits = [v for k, v in funcs.items() if k.startswith(pre)]
    if len(hits) != 1:
        raise RuntimeError("kernel %s: %d matches" % (kernel, len(hits)))
    return hits[0]


class RefDeviceRun:
    """The reference's device state (AoS particles, double3 buffers, cell_vec/nocup_vec) for one
    flume, resident on cuda:0, stepped by the reference's own kernels on `stream` (a CUDA stream
    handle; default: PyTorch's current stream)."""

    def __init__(self, sys, fun, cp, pp: np.ndarray, stream: int | None = None, min_margin: float = 0.25):
        import torch
        if not available():
            raise RuntimeError("reference device kernels not built (oracle/build.py builds them)")
        self.sys = np.array(sys, dtype=SYSTEM_PAR).reshape(()).copy()
        self.fun = np.array(fun, dtype=FUNNEL).reshape(()).copy()
        self.cp = np.array(cp, dtype=CELL_PAR).reshape(()).copy()
        pp = np.ascontiguousarray(pp, dtype=PARTICLE)
        self.n = len(pp)
        if int(self.sys["npart"]) != self.n:
            raise ValueError("system_par npart != len(pp)")
        m = grid_margin(pp, self.cp, self.sys)
        occ = max_occupancy(pp, self.cp, self.sys)
        if not m >= min_margin or 2 * occ > int(self.cp["ntags"]):
            raise ValueError("state not safely inside the grid: margin %.3g cells, fullest cell %d of %d slots"
                             % (m, occ, int(self.cp["ntags"])))
        self.drv = _Driver()
        self.mods = {}
        self.fn = {}
        for k, (mname, _) in KERNELS.items():
            if mname not in self.mods:
                self.mods[mname] = self.drv.load(os.path.join(DEV_DIR, mname + ".cubin"))
            self.fn[k] = _find(self.mods[mname][1], k)
        dev = torch.device("cuda")
        n = max(self.n, 1)
        self.t_pp = torch.from_numpy(pp.view(np.uint8).copy()).to(dev)
        self.t_vec = torch.zeros((6, n, 3), dtype=torch.float64, device=dev)   # F, T, a_i, al_i, a_f, al_f
        ntot, ncell3 = int(self.cp["ntot"]), int(self.cp["ncell3"])
        if ntot != ncell3 * int(self.cp["ntags"]):
            raise ValueError("cell_par ntot != ncell3 ntags")
        self.t_cell = torch.empty(max(ntot, 1), dtype=torch.int64, device=dev)
        self.t_ocup = torch.empty(max(ncell3, 1), dtype=torch.int32, device=dev)
        self.stream = C.c_void_p(stream if stream is not None else torch.cuda.current_stream().cuda_stream)
        self.rb_part = 1 + (self.n - 1) // NTHREAD
        self.rb_cell = 1 + (ntot - 1) // NTHREAD
        self.rb_ocup = 1 + (ncell3 - 1) // NTHREAD
        self.launches = 0
        self._order = [2, 3, 4, 5]   # slots of a_i, al_i, a_f, al_f in t_vec

    # ---- buffers ----
    def _ptr(self, t) -> int:
        return t.data_ptr()

    @property
    def F(self): return self._ptr(self.t_vec[0])
    @property
    def T(self): return self._ptr(self.t_vec[1])
    @property
    def a_i(self): return self._ptr(self.t_vec[self._order[0]])
    @property
    def al_i(self): return self._ptr(self.t_vec[self._order[1]])
    @property
    def a_f(self): return self._ptr(self.t_vec[self._order[2]])
    @property
    def al_f(self): return self._ptr(self.t_vec[self._order[3]])
    @property
    def pp(self): return self._ptr(self.t_pp)

    def set_accel(self, acc: np.ndarray, anga: np.ndarray) -> None:
        import torch
        self.t_vec[self._order[0]].copy_(torch.from_numpy(np.ascontiguousarray(acc, dtype=np.float64)))
        self.t_vec[self._order[1]].copy_(torch.from_numpy(np.ascontiguousarray(anga, dtype=np.float64)))

    def export(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        pp = self.t_pp.cpu().numpy().view(PARTICLE).copy()
        return pp, self.t_vec[self._order[0]].cpu().numpy().copy(), self.t_vec[self._order[1]].cpu().numpy().copy()

    # ---- launches ----
    def _launch(self, kernel: str, grid: int, *args) -> None:
        kinds = KERNELS[kernel][1]
        assert len(kinds) == len(args), kernel
        keep, params = [], []
        for kind, a in zip(kinds, args):
            if kind == "P":
                v = C.c_void_p(int(a))
            elif kind in "scf":
                v = np.array(a, copy=True)    # the struct's bytes, copied at launch
                keep.append(v)
                params.append(v.ctypes.data)
                continue
            elif kind == "b":
                v = C.c_char(bytes([int(a)]))
            else:
                v = C.c_int(int(a))
            keep.append(v)
            params.append(C.addressof(v))
        arr = (C.c_void_p * len(params))(*params)
        self.drv.check(self.drv.cu.cuLaunchKernel(self.fn[kernel], grid, 1, 1, NTHREAD, 1, 1, 0, self.stream,
                                                  arr, None), kernel)
        self.launches += 1

    def _cells(self) -> None:
        self._launch("clear_cell_dev", self.rb_cell, self.cp, self._ptr(self.t_cell))
        self._launch("clear_ocup_dev", self.rb_ocup, self.cp, self._ptr(self.t_ocup))
        self._launch("cell_locate_dev", self.rb_part, self.cp, self.sys, self.pp, self._ptr(self.t_ocup),
                     self._ptr(self.t_cell))

    def _part(self) -> None:
        for ii in range(1, 17):
            self._launch("force_part_dev", self.rb_part, self.F, self.T, self._ptr(self.t_cell),
                         self._ptr(self.t_ocup), self.pp, self.sys, self.cp, ii)

    def seed_accel(self) -> None:
        """a_i from the reference's device start-up pass (avalanche_dev.cu:335-360)."""
        if self.n == 0:
            return
        self._launch("clear_forces_dev", self.rb_part, self.sys, self.F, self.T)
        self._cells()
        self._part()
        for ii in range(3):
            self._launch("force_hop_dev", self.rb_part, self.F, self.T, self.sys, self.pp, ii)
        self._launch("get_accel_dev", self.rb_part, self.F, self.T, self.a_i, self.al_i, self.sys, self.pp)

    def step(self, k: int = 1) -> None:
        """k steps of avalanche_dev.cu:636-693 (the avalanche phase)."""
        for _ in range(k):
            if self.n == 0:
                self.sys["time"] = self.sys["time"] + self.sys["dt"]
                continue
            self._launch("init_Verlet_dev", self.rb_part, self.a_i, self.al_i, self.sys, self.pp)
            self.sys["time"] = self.sys["time"] + self.sys["dt"]
            self._launch("rotate_vectors_dev", self.rb_part, self.pp, self.sys)
            self._launch("clear_forces_dev", self.rb_part, self.sys, self.F, self.T)
            self._cells()
            for ii in range(3):
                self._launch("force_hop_dev", self.rb_part, self.F, self.T, self.sys, self.pp, ii)
            self._launch("force_funnel_dev", self.rb_part, self.F, self.T, self.sys, self.pp, self.fun)
            self._launch("force_fcorners_dev", self.rb_part, self.F, self.T, self.sys, self.fun, self.pp)
            self._launch("force_walls_dev", self.rb_part, self.F, self.T, self.sys, self.pp)
            self._part()
            self._launch("force_flume_dev", self.rb_part, self.F, self.T, self.sys, self.pp)
            self._launch("get_accel_dev", self.rb_part, self.F, self.T, self.a_f, self.al_f, self.sys, self.pp)
            self._launch("finish_Verlet_dev", self.rb_part, self.a_i, self.al_i, self.a_f, self.al_f, self.sys,
                         self.pp)
            o = self._order
            self._order = [o[2], o[3], o[0], o[1]]

    def check_next_step(self, min_margin: float = 0.25) -> None:
        """Raises unless the next step's cell_locate_dev stays inside cell_vec: the positions
        init_Verlet_dev will predict (r + dt (v + dt/2 a_i), init_Verlet.cu:36-43) are at least
        min_margin cells inside the grid and no cell receives more than half of ntags clumps."""
        pp, a, _ = self.export()
        dt = float(self.sys["dt"])
        q = pp.copy()
        q["rr"] = pp["rr"] + dt * (pp["vv"] + (0.5 * dt) * a)
        s = self.sys.copy()
        s["time"] = s["time"] + s["dt"]
        m, occ = grid_margin(q, self.cp, s), max_occupancy(q, self.cp, s)
        if not (m >= min_margin and 2 * occ <= int(self.cp["ntags"])):
            raise RuntimeError("next step would leave the grid: margin %.3g cells, fullest cell %d of %d slots"
                               % (m, occ, int(self.cp["ntags"])))

    def step_checked(self, k: int, min_margin: float = 0.25) -> None:
        """k steps, each after check_next_step."""
        for _ in range(k):
            self.check_next_step(min_margin)
            self.step(1)

    def snapshot(self):
        return self.t_pp.clone(), self.t_vec.clone(), self.sys.copy(), list(self._order)

    def restore(self, snap) -> None:
        self.t_pp.copy_(snap[0])
        self.t_vec.copy_(snap[1])
        self.sys = snap[2].copy()
        self._order = list(snap[3])

    def close(self) -> None:
        for mod, _ in self.mods.values():
            self.drv.cu.cuModuleUnload(mod)
        self.mods = {}
