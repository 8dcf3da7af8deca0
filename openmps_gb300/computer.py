"""Python mirror of OpenMps's ``Computer`` over the C ABI of ``libopenmps_gb300.so``.

``Computer`` follows the reference class (src/OpenMps/Computer.hpp:434-1790):
construct from the environment constants and the CG tolerance
(``CreateComputer``, :1800-1815), ``add_particles`` (``AddParticles``, :1754-1777),
``forward_time(dt)`` / ``forward_time()`` (``ForwardTime``, :1700-1751),
``particles()`` (``Particles``, :1780-1783) and ``environment()``
(``GetEnvironment``, :1786-1789).  Failures raise ``ComputerError`` carrying the
status code, as the reference raises ``Computer::Exception`` / ``Grid::Exception``.

Every call goes through the CUDA library; there is no CPU fallback.  Loading fails
loudly if the library has not been built (``openmps_gb300.build.build()``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi as abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libopenmps_gb300.so")
_LIB = None

_D = C.POINTER(C.c_double)
_F = C.POINTER(C.c_float)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)
_P = C.c_void_p

# every entry point of include/mps.h with its ctypes signature
PROTOTYPES = {
    "mps_default_params": (None, [C.POINTER(abi.MpsParams)]),
    "mps_params_size": (C.c_size_t, []),
    "mps_stats_size": (C.c_size_t, []),
    "mps_environment_size": (C.c_size_t, []),
    "mps_status_string": (C.c_char_p, [C.c_int]),
    "mps_last_error": (C.c_char_p, [_P]),
    "mps_version": (C.c_char_p, []),
    "mps_create": (C.c_int, [C.POINTER(abi.MpsParams), C.c_int, C.POINTER(_P)]),
    "mps_destroy": (C.c_int, [_P]),
    "mps_add_particles": (C.c_int, [_P, C.c_int64, _I32, _D, _D, _D, _D, _D, _D]),
    "mps_particle_count": (C.c_int64, [_P]),
    "mps_get_particles": (C.c_int, [_P, _I32, _D, _D, _D, _D, _D, _D]),
    "mps_set_particles": (C.c_int, [_P, _I32, _D, _D, _D, _D, _D, _D]),
    "mps_get_particles_device": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "mps_set_particles_device": (C.c_int, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "mps_set_wall_positions": (C.c_int, [_P, _D, _D]),
    "mps_add_particles3": (C.c_int, [_P, C.c_int64, _I32, _D, _D, _D, _D, _D, _D, _D, _D]),
    "mps_get_particles3": (C.c_int, [_P, _I32, _D, _D, _D, _D, _D, _D, _D, _D]),
    "mps_set_particles3": (C.c_int, [_P, _I32, _D, _D, _D, _D, _D, _D, _D, _D]),
    "mps_set_wall_positions3": (C.c_int, [_P, _D, _D, _D]),
    "mps_debug_get_aux3": (C.c_int, [_P, _D, _D, _D, _D, _D]),
    "mps_debug_set_aux3": (C.c_int, [_P, _D, _D, _D, _D, _D]),
    "mps_forward_time": (C.c_int, [_P, C.c_double]),
    "mps_forward_steps": (C.c_int, [_P, C.c_double, C.c_int32]),
    "mps_determine_dt": (C.c_int, [_P, _D]),
    "mps_debug_exact_arith": (C.c_int, [C.c_int32, C.c_int64, _D, _D, _D, _D]),
    "mps_get_environment": (C.c_int, [_P, C.POINTER(abi.MpsEnvironment)]),
    "mps_get_stats": (C.c_int, [_P, C.POINTER(abi.MpsStats)]),
    "mps_set_solver": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_double]),
    "mps_set_stage_timing": (C.c_int, [_P, C.c_int32]),
    "mps_set_wait_limits": (C.c_int, [_P, C.c_int64, C.c_int64]),
    "mps_synchronize": (C.c_int, [_P]),
    "mps_event_record": (C.c_int, [_P, C.c_int32]),
    "mps_event_elapsed": (C.c_int, [_P, C.c_int32, C.c_int32, C.POINTER(C.c_float)]),
    "mps_flush_l2": (C.c_int, [_P, C.c_int64]),
    "mps_bench_spmv": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int64, C.POINTER(C.c_float)]),
    "mps_spmv_bytes": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_int64)]),
    "mps_stage_search_neighbor": (C.c_int, [_P]),
    "mps_stage_density": (C.c_int, [_P]),
    "mps_stage_error_correction": (C.c_int, [_P]),
    "mps_stage_explicit": (C.c_int, [_P]),
    "mps_stage_save_x": (C.c_int, [_P]),
    "mps_stage_set_ppe": (C.c_int, [_P]),
    "mps_stage_solve_ppe": (C.c_int, [_P]),
    "mps_stage_assign_pressure": (C.c_int, [_P]),
    "mps_stage_pressure_gradient": (C.c_int, [_P]),
    "mps_stage_dynamic_stabilize": (C.c_int, [_P]),
    "mps_stage_begin_step": (C.c_int, [_P, C.c_double]),
    "mps_stage_density_variation": (C.c_int, [_P, _D]),
    "mps_debug_get_neighbors": (C.c_int, [_P, _I32, _I32, C.c_int64, _I64]),
    "mps_debug_get_ppe": (C.c_int, [_P, _I64, _I32, _D, _D, _D, C.c_int64, _I64]),
    "mps_debug_get_aux": (C.c_int, [_P, _D, _D, _D, _D]),
    "mps_debug_set_aux": (C.c_int, [_P, _D, _D, _D, _D]),
    "mps_cg_solve_csr": (C.c_int, [_P, C.c_int64, _I64, _I32, _D, _D, _D, C.c_double, C.c_int32,
                                   C.c_int32, C.c_int32, _I32, _D]),
    "mps_cg_solve_csr_device_noalloc": (C.c_int, [C.c_int64, _P, _P, _P, _P, _P, C.c_double,
                                                  C.c_int32, C.c_int32, _P, _I32, _D]),
    "mps_learned_set_weights": (C.c_int, [_P, _F, C.c_int64]),
    "mps_learned_collect": (C.c_int, [_P, C.c_int32]),
    "mps_learned_samples": (C.c_int, [_P, _F, _I32, C.c_int64, _I64]),
    "mps_mlp_infer": (C.c_int, [C.c_int32, _F, _F, C.c_int64, _F]),
    "mps_mlp_loss_grad": (C.c_int, [C.c_int32, _F, _F, C.c_int64, _F, _D]),
    "mps_mlp_train": (C.c_int, [C.c_int32, _F, _F, C.c_int64, C.c_int32, C.c_int32, C.c_float,
                                C.c_uint64, _D]),
    "mps_batch_create": (C.c_int, [C.POINTER(abi.MpsParams), C.c_int, C.c_int32, _I64, C.POINTER(_P)]),
    "mps_batch_set_scene": (C.c_int, [_P, C.c_int32, _I32, _D, _D, _D, _D, _D, _D]),
    "mps_batch_get_scene": (C.c_int, [_P, C.c_int32, _I32, _D, _D, _D, _D, _D, _D]),
    "mps_batch_forward": (C.c_int, [_P, C.c_double, C.c_int32]),
    "mps_batch_get_scene_stats": (C.c_int, [_P, C.c_int32, C.POINTER(abi.MpsBatchSceneStats)]),
    "mps_batch_tuning_info": (C.c_int, [_P, C.POINTER(abi.MpsBatchTuning)]),
}


def load_library(path: str | None = None) -> C.CDLL:
    """Loads ``libopenmps_gb300.so`` (raises if it is missing: no fallback exists)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            "libopenmps_gb300.so is not built (%s); run openmps_gb300.build.build() "
            "with the CUDA toolkit (there is no CPU fallback)" % p)
    lib = C.CDLL(p)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.mps_params_size() != C.sizeof(abi.MpsParams):
        raise RuntimeError("mps_params layout mismatch between mps.h and _abi.py")
    if lib.mps_stats_size() != C.sizeof(abi.MpsStats):
        raise RuntimeError("mps_stats layout mismatch between mps.h and _abi.py")
    if lib.mps_environment_size() != C.sizeof(abi.MpsEnvironment):
        raise RuntimeError("mps_environment layout mismatch between mps.h and _abi.py")
    if path is None:
        _LIB = lib
    return lib


class ComputerError(RuntimeError):
    """A failing status of the C ABI (the reference's Computer/Grid exceptions)."""

    def __init__(self, code: int, msg: str):
        super().__init__("status %d (%s): %s" % (code, _status_name(code), msg))
        self.code = code


def _status_name(code: int) -> str:
    try:
        return load_library().mps_status_string(code).decode()
    except Exception:  # pragma: no cover - only used for messages
        return "?"


def _ptr(a, ctype=C.c_double):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class Computer:
    """One scene on one GPU (``Computer<POSITION_WALL, POSITION_WALL_PRE>``)."""

    def __init__(self, params: abi.MpsParams, device: int = 0):
        self.lib = load_library()
        self.params = params
        h = C.c_void_p()
        rc = self.lib.mps_create(C.byref(params), device, C.byref(h))
        if rc:
            raise ComputerError(rc, "mps_create")
        self.h = h

    def close(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.mps_destroy(h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc:
            raise ComputerError(rc, self.lib.mps_last_error(self.h).decode())

    # ------------------------------------------------------------ particles
    def add_particles(self, t, x, z, u=None, w=None, p=None, n=None):
        t = np.ascontiguousarray(t, dtype=np.int32)
        arrs = [_f64(a) for a in (x, z, u, w, p, n)]
        self._check(self.lib.mps_add_particles(self.h, len(t), _ptr(t, C.c_int32),
                                               *[_ptr(a) for a in arrs]))

    def add_scene(self, scene):
        """Adds a ``scenes.Scene`` (2D) or ``scenes.Scene3`` (3D handle) particle set."""
        if hasattr(scene, "arrays3"):
            self.add_particles3(*scene.arrays3())
        else:
            self.add_particles(*scene.arrays())

    @property
    def count(self) -> int:
        return int(self.lib.mps_particle_count(self.h))

    def particles(self) -> dict:
        n = self.count
        out = {k: np.empty(n) for k in ("x", "z", "u", "w", "p", "n")}
        out["type"] = np.empty(n, dtype=np.int32)
        self._check(self.lib.mps_get_particles(self.h, _ptr(out["type"], C.c_int32),
                                               *[_ptr(out[k]) for k in ("x", "z", "u", "w", "p", "n")]))
        return out

    def get_particles_into(self, type_, x, z, u, w, p, n):
        """Copies the state into preallocated host arrays (any may be None)."""
        self._check(self.lib.mps_get_particles(self.h, _ptr(type_, C.c_int32), _ptr(x), _ptr(z),
                                               _ptr(u), _ptr(w), _ptr(p), _ptr(n)))

    def set_particles(self, t=None, x=None, z=None, u=None, w=None, p=None, n=None):
        t = None if t is None else np.ascontiguousarray(t, dtype=np.int32)
        self._check(self.lib.mps_set_particles(self.h, _ptr(t, C.c_int32),
                                               *[_ptr(_f64(a)) for a in (x, z, u, w, p, n)]))

    def set_wall_positions(self, wx, wz):
        self._check(self.lib.mps_set_wall_positions(self.h, _ptr(_f64(wx)), _ptr(_f64(wz))))

    # ------------------------------------------- three-dimensional scenes (dim = 3)
    FIELDS3 = ("x", "y", "z", "u", "v", "w", "p", "n")

    def add_particles3(self, t, x, y, z, u=None, v=None, w=None, p=None, n=None):
        t = np.ascontiguousarray(t, dtype=np.int32)
        arrs = [_f64(a) for a in (x, y, z, u, v, w, p, n)]
        self._check(self.lib.mps_add_particles3(self.h, len(t), _ptr(t, C.c_int32),
                                                *[_ptr(a) for a in arrs]))

    def particles3(self) -> dict:
        n = self.count
        out = {k: np.empty(n) for k in self.FIELDS3}
        out["type"] = np.empty(n, dtype=np.int32)
        self._check(self.lib.mps_get_particles3(self.h, _ptr(out["type"], C.c_int32),
                                                *[_ptr(out[k]) for k in self.FIELDS3]))
        return out

    def set_particles3(self, t=None, x=None, y=None, z=None, u=None, v=None, w=None, p=None, n=None):
        t = None if t is None else np.ascontiguousarray(t, dtype=np.int32)
        self._check(self.lib.mps_set_particles3(self.h, _ptr(t, C.c_int32),
                                                *[_ptr(_f64(a)) for a in (x, y, z, u, v, w, p, n)]))

    def set_wall_positions3(self, wx, wy, wz):
        self._check(self.lib.mps_set_wall_positions3(self.h, _ptr(_f64(wx)), _ptr(_f64(wy)), _ptr(_f64(wz))))

    def aux3(self) -> dict:
        n = self.count
        out = {k: np.zeros(n) for k in ("n_without_spp", "ecs", "ox", "oy", "oz")}
        self._check(self.lib.mps_debug_get_aux3(self.h, *[_ptr(out[k]) for k in
                                                          ("n_without_spp", "ecs", "ox", "oy", "oz")]))
        return out

    def set_aux3(self, n_without_spp=None, ecs=None, ox=None, oy=None, oz=None):
        self._check(self.lib.mps_debug_set_aux3(self.h, *[_ptr(_f64(a)) for a in
                                                          (n_without_spp, ecs, ox, oy, oz)]))

    # ---------------------------------------------------------------- steps
    def forward_time(self, dt: float | None = None):
        """``ForwardTime(dt)``; ``dt=None`` is ``ForwardTime()`` with the CFL time step."""
        self._check(self.lib.mps_forward_time(self.h, -1.0 if dt is None else float(dt)))

    def determine_dt(self) -> float:
        """The CFL time step ``ForwardTime()`` would take from the current state."""
        dt = C.c_double()
        self._check(self.lib.mps_determine_dt(self.h, C.byref(dt)))
        return float(dt.value)

    def forward_steps(self, dt: float, nsteps: int):
        self._check(self.lib.mps_forward_steps(self.h, float(dt), int(nsteps)))

    def environment(self) -> abi.MpsEnvironment:
        env = abi.MpsEnvironment()
        self._check(self.lib.mps_get_environment(self.h, C.byref(env)))
        return env

    def stats(self) -> dict:
        st = abi.MpsStats()
        self._check(self.lib.mps_get_stats(self.h, C.byref(st)))
        out = {name: getattr(st, name) for name, _ in abi.MpsStats._fields_ if name != "stage_ms"}
        out["stage_ms"] = dict(zip(abi.STAGE_NAMES, list(st.stage_ms)))
        return out

    def set_solver(self, solver: int, criterion: int, eps: float):
        self._check(self.lib.mps_set_solver(self.h, solver, criterion, eps))

    def set_stage_timing(self, enable: bool):
        self._check(self.lib.mps_set_stage_timing(self.h, 1 if enable else 0))

    def set_wait_limits(self, barrier_clocks: int = -1, mma_clocks: int = -1):
        """Bounds of the device-side waits in SM clocks (negative: the default)."""
        self._check(self.lib.mps_set_wait_limits(self.h, barrier_clocks, mma_clocks))

    # --------------------------------------------------------------- timing
    def synchronize(self):
        self._check(self.lib.mps_synchronize(self.h))

    def event_record(self, slot: int):
        self._check(self.lib.mps_event_record(self.h, slot))

    def event_elapsed(self, begin: int, end: int) -> float:
        ms = C.c_float()
        self._check(self.lib.mps_event_elapsed(self.h, begin, end, C.byref(ms)))
        return float(ms.value)

    def spmv_bytes(self, solver: int) -> int:
        """Algorithmic bytes of one launch of the solver's SpMV on the last matrix."""
        b = C.c_int64()
        self._check(self.lib.mps_spmv_bytes(self.h, solver, C.byref(b)))
        return int(b.value)

    def flush_l2(self, nbytes: int = 512 << 20):
        self._check(self.lib.mps_flush_l2(self.h, nbytes))

    def bench_spmv(self, solver: int, reps: int = 20, flush_bytes: int = 0) -> float:
        """Mean milliseconds of one launch of the solver's SpMV kernel."""
        ms = C.c_float()
        self._check(self.lib.mps_bench_spmv(self.h, solver, reps, flush_bytes, C.byref(ms)))
        return float(ms.value)

    # --------------------------------------------------------------- stages
    def stage(self, name: str):
        self._check(getattr(self.lib, "mps_stage_" + name)(self.h))

    def begin_step(self, dt: float):
        self._check(self.lib.mps_stage_begin_step(self.h, dt))

    def density_variation(self) -> np.ndarray:
        out = np.zeros(self.count)
        self._check(self.lib.mps_stage_density_variation(self.h, _ptr(out)))
        return out

    def neighbors(self):
        n = self.count
        counts = np.zeros(n, dtype=np.int32)
        total = C.c_int64()
        self._check(self.lib.mps_debug_get_neighbors(self.h, _ptr(counts, C.c_int32), None, 0,
                                                     C.byref(total)))
        lst = np.zeros(max(total.value, 1), dtype=np.int32)
        self._check(self.lib.mps_debug_get_neighbors(self.h, _ptr(counts, C.c_int32),
                                                     _ptr(lst, C.c_int32), lst.size, C.byref(total)))
        return counts, lst[: total.value]

    def ppe(self):
        n = self.count
        nnz = C.c_int64()
        rp = np.zeros(n + 1, dtype=np.int64)
        self._check(self.lib.mps_debug_get_ppe(self.h, _ptr(rp, C.c_int64), None, None, None, None,
                                               0, C.byref(nnz)))
        col = np.zeros(max(nnz.value, 1), dtype=np.int32)
        val = np.zeros(max(nnz.value, 1))
        b = np.zeros(n)
        x = np.zeros(n)
        self._check(self.lib.mps_debug_get_ppe(self.h, _ptr(rp, C.c_int64), _ptr(col, C.c_int32),
                                               _ptr(val), _ptr(b), _ptr(x), col.size, C.byref(nnz)))
        return rp, col[: nnz.value], val[: nnz.value], b, x

    def aux(self) -> dict:
        n = self.count
        out = {k: np.zeros(n) for k in ("n_without_spp", "ecs", "ox", "oz")}
        self._check(self.lib.mps_debug_get_aux(self.h, *[_ptr(out[k]) for k in
                                                         ("n_without_spp", "ecs", "ox", "oz")]))
        return out

    def set_aux(self, n_without_spp=None, ecs=None, ox=None, oz=None):
        self._check(self.lib.mps_debug_set_aux(self.h, *[_ptr(_f64(a)) for a in
                                                         (n_without_spp, ecs, ox, oz)]))

    # ---------------------------------------------------------- learned solve
    def learned_set_weights(self, blob):
        w = _f32(blob)
        self._check(self.lib.mps_learned_set_weights(self.h, _ptr(w, C.c_float), w.size))

    def learned_collect(self, enable: bool):
        self._check(self.lib.mps_learned_collect(self.h, 1 if enable else 0))

    def learned_samples(self):
        """The last step's (n, 18) samples and (n,) active-row flags."""
        n = self.count
        out = np.zeros((n, abi.MLP_SAMPLE_FLOATS), dtype=np.float32)
        act = np.zeros(n, dtype=np.int32)
        cnt = C.c_int64()
        self._check(self.lib.mps_learned_samples(self.h, _ptr(out, C.c_float), _ptr(act, C.c_int32), n,
                                                 C.byref(cnt)))
        return out, act

    def cg_solve_csr(self, row_ptr, col, val, b, x0, eps, criterion=abi.CRIT_INITIAL_RESIDUAL,
                     max_iters=0, solver=abi.SOLVER_CG64):
        """SolvePressurePoissonEquation on a caller CSR system; returns (x, iterations, relres)."""
        rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
        cl = np.ascontiguousarray(col, dtype=np.int32)
        va = _f64(val)
        bb = _f64(b)
        x = np.array(x0, dtype=np.float64, copy=True)
        it = C.c_int32()
        rel = C.c_double()
        self._check(self.lib.mps_cg_solve_csr(self.h, len(bb), _ptr(rp, C.c_int64), _ptr(cl, C.c_int32),
                                              _ptr(va), _ptr(bb), _ptr(x), eps, criterion, max_iters,
                                              solver, C.byref(it), C.byref(rel)))
        return x, it.value, rel.value


class Batch(Computer):
    """Independent scenes sharing one parameter set, advanced together (mps_batch_*).

    Each scene behaves like its own ``Computer``; ``forward(dt, nsteps)`` advances all of
    them with a fixed dt (the first step autotunes the batched PPE solve, later steps
    replay one captured CUDA graph per step).
    """

    def __init__(self, params: abi.MpsParams, scenes, device: int = 0):
        self.lib = load_library()
        self.h = None
        counts = np.array([s.count for s in scenes], dtype=np.int64)
        h = C.c_void_p()
        rc = self.lib.mps_batch_create(C.byref(params), device, len(scenes), _ptr(counts, C.c_int64),
                                       C.byref(h))
        if rc != abi.MPS_OK:
            raise ComputerError(rc, "mps_batch_create")
        self.h = h
        self.params = params
        self.counts = counts
        for k, s in enumerate(scenes):
            self._check(self.lib.mps_batch_set_scene(self.h, k, _ptr(np.ascontiguousarray(s.type, np.int32), C.c_int32),
                                                     *[_ptr(_f64(a)) for a in (s.x, s.z, s.u, s.w, s.p, s.n)]))

    def forward(self, dt: float, nsteps: int = 1):
        self._check(self.lib.mps_batch_forward(self.h, dt, nsteps))

    def scene(self, k: int) -> dict:
        n = int(self.counts[k])
        out = {"type": np.zeros(n, dtype=np.int32)}
        for key in ("x", "z", "u", "w", "p", "n"):
            out[key] = np.zeros(n)
        self._check(self.lib.mps_batch_get_scene(self.h, k, _ptr(out["type"], C.c_int32),
                                                 *[_ptr(out[key]) for key in ("x", "z", "u", "w", "p", "n")]))
        return out

    def scene_stats(self, k: int) -> dict:
        st = abi.MpsBatchSceneStats()
        self._check(self.lib.mps_batch_get_scene_stats(self.h, k, C.byref(st)))
        return {name: getattr(st, name) for name, _ in abi.MpsBatchSceneStats._fields_ if name != "pad"}

    def tuning(self) -> dict:
        t = abi.MpsBatchTuning()
        self._check(self.lib.mps_batch_tuning_info(self.h, C.byref(t)))
        n = t.candidates
        return {"threads": t.threads, "blocks": t.blocks, "order": t.order,
                "candidates": [{"threads": t.candidate_threads[k], "order": t.candidate_order[k],
                                "ms": t.candidate_ms[k]} for k in range(n)]}


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _status(rc: int, what: str):
    if rc != abi.MPS_OK:
        raise ComputerError(rc, what)


def exact_arith(a, b, device: int = 0):
    """(a / b, sqrt(a)) by the stage kernels' FP64 division and square root on the GPU."""
    lib = load_library()
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    q = np.empty_like(a)
    r = np.empty_like(a)
    _status(lib.mps_debug_exact_arith(device, a.size, _ptr(a), _ptr(b), _ptr(q), _ptr(r)),
            "mps_debug_exact_arith")
    return q, r


def mlp_infer(blob, features, device: int = 0) -> np.ndarray:
    """Tensor-core inference of the learned-solve network: (n, 16) features -> (n, 2)."""
    lib = load_library()
    w = _f32(blob)
    f = _f32(features)
    n = f.shape[0]
    out = np.zeros((n, 2), dtype=np.float32)
    _status(lib.mps_mlp_infer(device, _ptr(w, C.c_float), _ptr(f, C.c_float), n, _ptr(out, C.c_float)),
            "mps_mlp_infer")
    return out


def mlp_loss_grad(blob, samples, device: int = 0):
    """(mean loss, gradient) of the learned-solve network on (n, 18) samples (GPU kernels)."""
    lib = load_library()
    w = _f32(blob)
    s = _f32(samples)
    grad = np.zeros(abi.MLP_BLOB_FLOATS, dtype=np.float32)
    loss = C.c_double()
    _status(lib.mps_mlp_loss_grad(device, _ptr(w, C.c_float), _ptr(s, C.c_float), s.shape[0],
                                  _ptr(grad, C.c_float), C.byref(loss)), "mps_mlp_loss_grad")
    return loss.value, grad


def mlp_train(blob, samples, epochs: int, batch: int = 4096, lr: float = 1e-3, seed: int = 0,
              device: int = 0):
    """Adam training on the GPU; returns (trained blob, mean loss per epoch)."""
    lib = load_library()
    w = np.array(blob, dtype=np.float32, copy=True)
    s = _f32(samples)
    losses = np.zeros(epochs)
    _status(lib.mps_mlp_train(device, _ptr(w, C.c_float), _ptr(s, C.c_float), s.shape[0], epochs,
                              batch, lr, seed, _ptr(losses)), "mps_mlp_train")
    return w, losses


def create_computer(eps: float, params: abi.MpsParams, device: int = 0) -> Computer:
    """``CreateComputer(allowableResidual, env, posWall, posWallPre)`` with static walls."""
    p = abi.MpsParams.from_buffer_copy(params)
    p.eps = eps
    return Computer(p, device)
