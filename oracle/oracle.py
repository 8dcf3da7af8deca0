"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this module.  It loads ``oracle/_build/libmps_oracle.so``
(serial parity oracle) or ``libmps_oracle_omp.so`` (OpenMP CPU baseline), both
built by ``oracle/build_oracle.py`` from ``mps_oracle.cpp``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from openmps_gb300 import _abi as abi

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS: dict[str, C.CDLL] = {}

_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)


def _ptr(a, ctype=C.c_double):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


def load(openmp: bool = False) -> C.CDLL:
    name = "libmps_oracle_omp.so" if openmp else "libmps_oracle.so"
    if name in _LIBS:
        return _LIBS[name]
    path = os.path.join(HERE, "_build", name)
    if not os.path.exists(path):
        from . import build_oracle  # noqa: WPS433 (local import keeps build optional)

        build_oracle.build()
    lib = C.CDLL(path)
    P = C.c_void_p
    lib.oracle_create.argtypes = [C.POINTER(abi.MpsParams), C.POINTER(P)]
    lib.oracle_destroy.argtypes = [P]
    lib.oracle_destroy.restype = None
    lib.oracle_last_error.argtypes = [P]
    lib.oracle_last_error.restype = C.c_char_p
    lib.oracle_add_particles.argtypes = [P, C.c_int64, _I32, _D, _D, _D, _D, _D, _D]
    lib.oracle_particle_count.argtypes = [P]
    lib.oracle_particle_count.restype = C.c_int64
    lib.oracle_get_particles.argtypes = [P, _I32, _D, _D, _D, _D, _D, _D]
    lib.oracle_set_particles.argtypes = [P, _I32, _D, _D, _D, _D, _D, _D]
    lib.oracle_set_wall_positions.argtypes = [P, _D, _D]
    lib.oracle_set_solver.argtypes = [P, C.c_int32, C.c_double, C.c_int32]
    lib.oracle_forward_time.argtypes = [P, C.c_double]
    lib.oracle_get_environment.argtypes = [P, C.POINTER(abi.MpsEnvironment)]
    lib.oracle_get_stats.argtypes = [P, _I32, _D, _D, _I64, _I64]
    for st in ("search_neighbor", "density", "error_correction", "explicit", "save_x", "set_ppe",
               "solve_ppe", "assign_pressure", "pressure_gradient", "dynamic_stabilize"):
        getattr(lib, "oracle_stage_" + st).argtypes = [P]
    lib.oracle_stage_begin_step.argtypes = [P, C.c_double]
    lib.oracle_stage_density_variation.argtypes = [P, _D]
    lib.oracle_determine_dt.argtypes = [P]
    lib.oracle_determine_dt.restype = C.c_double
    lib.oracle_get_neighbors.argtypes = [P, _I32, _I32, C.c_int64, _I64]
    lib.oracle_get_ppe.argtypes = [P, _I64, _I32, _D, _D, _D, C.c_int64, _I64]
    lib.oracle_set_ppe_x.argtypes = [P, _D]
    lib.oracle_get_aux.argtypes = [P, _D, _D, _D, _D]
    lib.oracle_set_aux.argtypes = [P, _D, _D, _D, _D]
    lib.oracle_cg_solve_csr.argtypes = [C.c_int64, _I64, _I32, _D, _D, _D, C.c_double, C.c_int32,
                                        C.c_int32, _I32, _D, _D]
    lib.oracle_num_threads.restype = C.c_int
    lib.oracle_gc_invert.argtypes = [_D, C.c_double, _D]
    lib.oracle_gc_invert.restype = None
    # three-dimensional oracle
    lib.oracle3_create.argtypes = [C.POINTER(abi.MpsParams), C.POINTER(P)]
    lib.oracle3_destroy.argtypes = [P]
    lib.oracle3_destroy.restype = None
    lib.oracle3_last_error.argtypes = [P]
    lib.oracle3_last_error.restype = C.c_char_p
    lib.oracle3_add_particles.argtypes = [P, C.c_int64, _I32] + [_D] * 8
    lib.oracle3_particle_count.argtypes = [P]
    lib.oracle3_particle_count.restype = C.c_int64
    lib.oracle3_get_particles.argtypes = [P, _I32] + [_D] * 8
    lib.oracle3_set_particles.argtypes = [P, _I32] + [_D] * 8
    lib.oracle3_forward_time.argtypes = [P, C.c_double]
    lib.oracle3_set_wall_positions.argtypes = [P, _D, _D, _D]
    lib.oracle3_get_environment.argtypes = [P, C.POINTER(abi.MpsEnvironment)]
    lib.oracle3_stage.argtypes = [P, C.c_int32, C.c_double]
    lib.oracle3_density_variation.argtypes = [P, _D]
    lib.oracle3_get_neighbors.argtypes = [P, _I32, _I32, C.c_int64, _I64]
    lib.oracle3_get_ppe.argtypes = [P, _I64, _I32, _D, _D, _D, C.c_int64, _I64]
    lib.oracle3_get_aux.argtypes = [P] + [_D] * 5
    lib.oracle3_set_aux.argtypes = [P] + [_D] * 5
    lib.oracle3_get_stats.argtypes = [P, _I32]
    lib.oracle3_gc_invert.argtypes = [_D, C.c_double, _D]
    lib.oracle3_gc_invert.restype = None
    _LIBS[name] = lib
    return lib


class OracleError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("oracle status %d: %s" % (code, msg))
        self.code = code


class Oracle:
    """CPU restatement of ``Computer`` (one scene)."""

    def __init__(self, params: abi.MpsParams, openmp: bool = False):
        self.lib = load(openmp)
        self.params = params
        h = C.c_void_p()
        rc = self.lib.oracle_create(C.byref(params), C.byref(h))
        if rc:
            raise OracleError(rc, "create")
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.oracle_destroy(h)
            self.h = None

    def _check(self, rc):
        if rc:
            raise OracleError(rc, self.lib.oracle_last_error(self.h).decode())

    # ---------------------------------------------------------------- state
    def add_particles(self, t, x, z, u=None, w=None, p=None, n=None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None
                for a in (x, z, u, w, p, n)]
        t = np.ascontiguousarray(t, dtype=np.int32)
        self._check(self.lib.oracle_add_particles(self.h, len(t), _ptr(t, C.c_int32),
                                                  *[_ptr(a) for a in arrs]))

    def add_scene(self, scene):
        self.add_particles(*scene.arrays())

    @property
    def count(self) -> int:
        return int(self.lib.oracle_particle_count(self.h))

    def particles(self) -> dict:
        n = self.count
        out = {k: np.empty(n) for k in ("x", "z", "u", "w", "p", "n")}
        out["type"] = np.empty(n, dtype=np.int32)
        self._check(self.lib.oracle_get_particles(self.h, _ptr(out["type"], C.c_int32),
                                                  *[_ptr(out[k]) for k in ("x", "z", "u", "w", "p", "n")]))
        return out

    def set_particles(self, t=None, x=None, z=None, u=None, w=None, p=None, n=None):
        conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        t = None if t is None else np.ascontiguousarray(t, dtype=np.int32)
        self._check(self.lib.oracle_set_particles(self.h, _ptr(t, C.c_int32),
                                                  *[_ptr(conv(a)) for a in (x, z, u, w, p, n)]))

    def set_wall_positions(self, wx, wz):
        self._check(self.lib.oracle_set_wall_positions(
            self.h, _ptr(np.ascontiguousarray(wx, dtype=np.float64)),
            _ptr(np.ascontiguousarray(wz, dtype=np.float64))))

    def set_solver(self, criterion: int, eps: float, max_iters: int = 0):
        self._check(self.lib.oracle_set_solver(self.h, criterion, eps, max_iters))

    def environment(self) -> abi.MpsEnvironment:
        env = abi.MpsEnvironment()
        self._check(self.lib.oracle_get_environment(self.h, C.byref(env)))
        return env

    def stats(self) -> dict:
        it = C.c_int32()
        rr0, rr = C.c_double(), C.c_double()
        nnz, nbt = C.c_int64(), C.c_int64()
        self._check(self.lib.oracle_get_stats(self.h, C.byref(it), C.byref(rr0), C.byref(rr),
                                              C.byref(nnz), C.byref(nbt)))
        return {"cg_iterations": it.value, "cg_rr0": rr0.value, "cg_rr": rr.value,
                "ppe_nnz": nnz.value, "neighbor_total": nbt.value}

    # ---------------------------------------------------------------- steps
    def forward_time(self, dt: float):
        self._check(self.lib.oracle_forward_time(self.h, dt))

    def stage(self, name: str, *args):
        self._check(getattr(self.lib, "oracle_stage_" + name)(self.h, *args))

    def begin_step(self, dt: float):
        self._check(self.lib.oracle_stage_begin_step(self.h, dt))

    def density_variation(self) -> np.ndarray:
        out = np.zeros(self.count)
        self._check(self.lib.oracle_stage_density_variation(self.h, _ptr(out)))
        return out

    def determine_dt(self) -> float:
        return float(self.lib.oracle_determine_dt(self.h))

    # ---------------------------------------------------------------- debug
    def neighbors(self):
        n = self.count
        counts = np.zeros(n, dtype=np.int32)
        total = C.c_int64()
        self._check(self.lib.oracle_get_neighbors(self.h, _ptr(counts, C.c_int32), None, 0,
                                                  C.byref(total)))
        lst = np.zeros(max(total.value, 1), dtype=np.int32)
        self._check(self.lib.oracle_get_neighbors(self.h, _ptr(counts, C.c_int32),
                                                  _ptr(lst, C.c_int32), lst.size, C.byref(total)))
        return counts, lst[: total.value]

    def ppe(self):
        n = self.count
        nnz = C.c_int64()
        rp = np.zeros(n + 1, dtype=np.int64)
        self._check(self.lib.oracle_get_ppe(self.h, _ptr(rp, C.c_int64), None, None, None, None, 0,
                                            C.byref(nnz)))
        col = np.zeros(max(nnz.value, 1), dtype=np.int32)
        val = np.zeros(max(nnz.value, 1))
        b = np.zeros(n)
        x = np.zeros(n)
        self._check(self.lib.oracle_get_ppe(self.h, _ptr(rp, C.c_int64), _ptr(col, C.c_int32),
                                            _ptr(val), _ptr(b), _ptr(x), col.size, C.byref(nnz)))
        return rp, col[: nnz.value], val[: nnz.value], b, x

    def set_ppe_x(self, x):
        self._check(self.lib.oracle_set_ppe_x(self.h, _ptr(np.ascontiguousarray(x, dtype=np.float64))))

    def aux(self) -> dict:
        n = self.count
        out = {k: np.zeros(n) for k in ("n_without_spp", "ecs", "ox", "oz")}
        self._check(self.lib.oracle_get_aux(self.h, *[_ptr(out[k]) for k in
                                                       ("n_without_spp", "ecs", "ox", "oz")]))
        return out

    def set_aux(self, n_without_spp=None, ecs=None, ox=None, oz=None):
        conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        self._check(self.lib.oracle_set_aux(self.h, *[_ptr(conv(a)) for a in
                                                      (n_without_spp, ecs, ox, oz)]))


def cg_solve_csr(row_ptr, col, val, b, x0, eps, criterion=abi.CRIT_INITIAL_RESIDUAL,
                 max_iters=0, openmp=False):
    """Reference CG on a CSR system. Returns (x, iterations, rr0, rr, status)."""
    lib = load(openmp)
    rp = np.ascontiguousarray(row_ptr, dtype=np.int64)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    va = np.ascontiguousarray(val, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.array(x0, dtype=np.float64, copy=True)
    it = C.c_int32()
    rr0, rr = C.c_double(), C.c_double()
    rc = lib.oracle_cg_solve_csr(len(bb), _ptr(rp, C.c_int64), _ptr(cl, C.c_int32), _ptr(va),
                                 _ptr(bb), _ptr(x), eps, criterion, max_iters, C.byref(it),
                                 C.byref(rr0), C.byref(rr))
    return x, it.value, rr0.value, rr.value, rc


def num_threads(openmp=True) -> int:
    return int(load(openmp).oracle_num_threads())


def gc_invert(m, val):
    """Detail::InvertMatrix<2> of the row-major 2x2 matrix m (4 values)."""
    a = np.ascontiguousarray(m, dtype=np.float64).reshape(4)
    out = np.zeros(4)
    load(False).oracle_gc_invert(_ptr(a), float(val), _ptr(out))
    return out


def gc_invert3(m, val):
    """Detail::InvertMatrix<3> of the row-major 3x3 matrix m (9 values)."""
    a = np.ascontiguousarray(m, dtype=np.float64).reshape(9)
    out = np.zeros(9)
    load(False).oracle3_gc_invert(_ptr(a), float(val), _ptr(out))
    return out


class Oracle3:
    """CPU restatement of the DIM3 build of ``Computer`` (one scene)."""

    FIELDS = ("x", "y", "z", "u", "v", "w", "p", "n")
    STAGES = {"search_neighbor": 1, "density": 2, "error_correction": 3, "explicit": 4, "save_x": 5,
              "set_ppe": 6, "solve_ppe": 7, "assign_pressure": 8, "pressure_gradient": 9,
              "dynamic_stabilize": 10}

    def __init__(self, params: abi.MpsParams, openmp: bool = False):
        self.lib = load(openmp)
        self.params = params
        h = C.c_void_p()
        rc = self.lib.oracle3_create(C.byref(params), C.byref(h))
        if rc:
            raise OracleError(rc, "create")
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.oracle3_destroy(h)
            self.h = None

    def _check(self, rc):
        if rc:
            raise OracleError(rc, self.lib.oracle3_last_error(self.h).decode())

    def add_particles(self, t, x, y, z, u=None, v=None, w=None, p=None, n=None):
        conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        t = np.ascontiguousarray(t, dtype=np.int32)
        self._check(self.lib.oracle3_add_particles(self.h, len(t), _ptr(t, C.c_int32),
                                                   *[_ptr(conv(a)) for a in (x, y, z, u, v, w, p, n)]))

    def add_scene(self, scene):
        self.add_particles(*scene.arrays3())

    @property
    def count(self) -> int:
        return int(self.lib.oracle3_particle_count(self.h))

    def particles(self) -> dict:
        n = self.count
        out = {k: np.empty(n) for k in self.FIELDS}
        out["type"] = np.empty(n, dtype=np.int32)
        self._check(self.lib.oracle3_get_particles(self.h, _ptr(out["type"], C.c_int32),
                                                   *[_ptr(out[k]) for k in self.FIELDS]))
        return out

    def set_particles(self, t=None, x=None, y=None, z=None, u=None, v=None, w=None, p=None, n=None):
        conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        t = None if t is None else np.ascontiguousarray(t, dtype=np.int32)
        self._check(self.lib.oracle3_set_particles(self.h, _ptr(t, C.c_int32),
                                                   *[_ptr(conv(a)) for a in (x, y, z, u, v, w, p, n)]))

    def forward_time(self, dt: float):
        self._check(self.lib.oracle3_forward_time(self.h, dt))

    def set_wall_positions(self, wx, wy, wz):
        conv = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self._check(self.lib.oracle3_set_wall_positions(self.h, _ptr(conv(wx)), _ptr(conv(wy)), _ptr(conv(wz))))

    def begin_step(self, dt: float):
        self._check(self.lib.oracle3_stage(self.h, 0, dt))

    def stage(self, name: str):
        self._check(self.lib.oracle3_stage(self.h, self.STAGES[name], 0.0))

    def environment(self) -> abi.MpsEnvironment:
        env = abi.MpsEnvironment()
        self._check(self.lib.oracle3_get_environment(self.h, C.byref(env)))
        return env

    def density_variation(self) -> np.ndarray:
        out = np.zeros(self.count)
        self._check(self.lib.oracle3_density_variation(self.h, _ptr(out)))
        return out

    def neighbors(self):
        n = self.count
        counts = np.zeros(n, dtype=np.int32)
        total = C.c_int64()
        self._check(self.lib.oracle3_get_neighbors(self.h, _ptr(counts, C.c_int32), None, 0, C.byref(total)))
        lst = np.zeros(max(total.value, 1), dtype=np.int32)
        self._check(self.lib.oracle3_get_neighbors(self.h, _ptr(counts, C.c_int32), _ptr(lst, C.c_int32),
                                                   lst.size, C.byref(total)))
        return counts, lst[: total.value]

    def ppe(self):
        n = self.count
        nnz = C.c_int64()
        rp = np.zeros(n + 1, dtype=np.int64)
        self._check(self.lib.oracle3_get_ppe(self.h, _ptr(rp, C.c_int64), None, None, None, None, 0,
                                             C.byref(nnz)))
        col = np.zeros(max(nnz.value, 1), dtype=np.int32)
        val = np.zeros(max(nnz.value, 1))
        b = np.zeros(n)
        x = np.zeros(n)
        self._check(self.lib.oracle3_get_ppe(self.h, _ptr(rp, C.c_int64), _ptr(col, C.c_int32), _ptr(val),
                                             _ptr(b), _ptr(x), col.size, C.byref(nnz)))
        return rp, col[: nnz.value], val[: nnz.value], b, x

    def aux(self) -> dict:
        n = self.count
        out = {k: np.zeros(n) for k in ("n_without_spp", "ecs", "ox", "oy", "oz")}
        self._check(self.lib.oracle3_get_aux(self.h, *[_ptr(out[k]) for k in
                                                       ("n_without_spp", "ecs", "ox", "oy", "oz")]))
        return out

    def set_aux(self, n_without_spp=None, ecs=None, ox=None, oy=None, oz=None):
        conv = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        self._check(self.lib.oracle3_set_aux(self.h, *[_ptr(conv(a)) for a in
                                                       (n_without_spp, ecs, ox, oy, oz)]))

    def stats(self) -> dict:
        it = C.c_int32()
        self._check(self.lib.oracle3_get_stats(self.h, C.byref(it)))
        return {"cg_iterations": it.value}
