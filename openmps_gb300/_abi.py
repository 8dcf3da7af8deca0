"""ctypes mirror of ``include/mps.h`` (structs, constants, prototypes).

The same struct layouts are used by the product library (``libopenmps_gb300.so``)
and by the test oracle, which includes ``mps.h`` for its parameter structs.
"""
from __future__ import annotations

import ctypes as C

# status codes
MPS_OK = 0
MPS_ERR_INVALID_ARGUMENT = 1
MPS_ERR_CUDA = 2
MPS_ERR_OUT_OF_MEMORY = 3
MPS_ERR_CELL_OVERFLOW = 4
MPS_ERR_CG_NOT_CONVERGED = 5
MPS_ERR_NOT_SUPPORTED = 6
MPS_ERR_STATE = 7
MPS_ERR_NONFINITE = 8
MPS_ERR_TIMEOUT = 9
MPS_ERR_DEVICE_CHECK = 10
MPS_ERR_NOALLOC_TOO_LARGE = 11
NOALLOC_MAX_ROWS = 262144

# particle types (src/OpenMps/Particle.hpp:16-29)
TYPE_FLUID = 0
TYPE_WALL = 1
TYPE_DUMMY = 2
TYPE_DISABLED = 3

# method flags (runtime form of src/OpenMps/defines.hpp:9-56)
FLAG_HS = 0x01
FLAG_HL = 0x02
FLAG_ECS = 0x04
FLAG_DS = 0x08
FLAG_SPP = 0x10
FLAG_GC = 0x20
FLAG_PRESSURE_EXPLICIT = 0x40
FLAG_CENTRAL_GRAVITY = 0x80
FLAGS_ALL = (FLAG_HS | FLAG_HL | FLAG_ECS | FLAG_DS | FLAG_SPP | FLAG_GC | FLAG_PRESSURE_EXPLICIT
             | FLAG_CENTRAL_GRAVITY)
PRESET_REFERENCE = FLAG_HS | FLAG_HL | FLAG_ECS | FLAG_DS | FLAG_SPP
PRESET_PLAIN = 0

SOLVER_CG64 = 0
SOLVER_MIXED = 1
SOLVER_LEARNED = 2
SOLVER_MIXED_MG = 3
SOLVER_NAMES = {SOLVER_CG64: "cg64", SOLVER_MIXED: "mixed", SOLVER_LEARNED: "learned",
                SOLVER_MIXED_MG: "mixed_mg"}

MLP_BLOB_FLOATS = 9570
MLP_SAMPLE_FLOATS = 18

CG_LAUNCH_GRAPH = 0
CG_LAUNCH_HOST = 1
CG_LAUNCH_GRAPH_KERNELS = 0
CG_LAUNCH_PERSISTENT = 2

CRIT_INITIAL_RESIDUAL = 0
CRIT_RHS = 1


class MpsParams(C.Structure):
    _fields_ = [
        ("max_dt", C.c_double),
        ("courant", C.c_double),
        ("g", C.c_double),
        ("rho", C.c_double),
        ("nu", C.c_double),
        ("surface_ratio", C.c_double),
        ("re_by_l0", C.c_double),
        ("re_lap_by_l0", C.c_double),
        ("l0", C.c_double),
        ("min_x", C.c_double),
        ("min_z", C.c_double),
        ("max_x", C.c_double),
        ("max_z", C.c_double),
        ("eps", C.c_double),
        ("flags", C.c_uint32),
        ("solver", C.c_int32),
        ("criterion", C.c_int32),
        ("max_cg_iters", C.c_int32),
        ("inner_tol", C.c_double),
        ("max_refinements", C.c_int32),
        ("cg_launch", C.c_int32),
        ("sound_speed", C.c_double),
        ("dim", C.c_int32),
        ("pad0", C.c_int32),
        ("min_y", C.c_double),
        ("max_y", C.c_double),
        ("reserved", C.c_double * 2),
    ]


class MpsEnvironment(C.Structure):
    _fields_ = [
        ("t", C.c_double),
        ("dt", C.c_double),
        ("n0", C.c_double),
        ("lambda_", C.c_double),
        ("n0_lap", C.c_double),
        ("lambda_lap", C.c_double),
        ("max_dt", C.c_double),
        ("max_dx", C.c_double),
        ("l0", C.c_double),
        ("re", C.c_double),
        ("re_lap", C.c_double),
        ("neighbor_length", C.c_double),
        ("rho", C.c_double),
        ("nu", C.c_double),
        ("g", C.c_double),
        ("min_x", C.c_double),
        ("min_z", C.c_double),
        ("max_x", C.c_double),
        ("max_z", C.c_double),
        ("grid_nx", C.c_int64),
        ("grid_nz", C.c_int64),
        ("grid_max_per_cell", C.c_int64),
        ("min_y", C.c_double),
        ("max_y", C.c_double),
        ("grid_ny", C.c_int64),
        ("dim", C.c_int64),
    ]


class MpsStats(C.Structure):
    _fields_ = [
        ("steps", C.c_int64),
        ("kernel_launches", C.c_int64),
        ("neighbor_total", C.c_int64),
        ("ppe_nnz", C.c_int64),
        ("cg_iterations", C.c_int32),
        ("cg_refinements", C.c_int32),
        ("disabled", C.c_int32),
        ("fallback", C.c_int32),
        ("cg_rr0", C.c_double),
        ("cg_rr", C.c_double),
        ("cg_true_relres", C.c_double),
        ("stage_ms", C.c_double * 12),
    ]


class MpsBatchSceneStats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32),
        ("reliable_updates", C.c_int32),
        ("fallback", C.c_int32),
        ("converged", C.c_int32),
        ("fallback_iterations", C.c_int32),
        ("pad", C.c_int32),
        ("true_relres", C.c_double),
        ("initial_relres", C.c_double),
    ]


class MpsBatchTuning(C.Structure):
    _fields_ = [
        ("threads", C.c_int32),
        ("blocks", C.c_int32),
        ("order", C.c_int32),
        ("candidates", C.c_int32),
        ("candidate_ms", C.c_float * 16),
        ("candidate_threads", C.c_int32 * 16),
        ("candidate_order", C.c_int32 * 16),
    ]


STAGE_NAMES = (
    "search", "density", "ecs", "explicit", "density2", "ppe", "solve", "pressure",
    "gradient", "ds", "other", "total",
)


def make_params(**kw) -> MpsParams:
    """Parameters with the reference's Sample.xml constants, overridden by ``kw``."""
    p = MpsParams()
    p.max_dt = 0.005 / 10
    p.courant = 0.1
    p.g = 9.8
    p.rho = 998.2
    p.nu = 1.004e-6
    p.surface_ratio = 0.97
    p.re_by_l0 = 2.4
    p.re_lap_by_l0 = 0.0
    p.l0 = 0.008
    p.min_x, p.min_z, p.max_x, p.max_z = -0.032, -0.032, 0.584, 0.584
    p.eps = 1e-10
    p.flags = PRESET_REFERENCE
    p.solver = SOLVER_CG64
    p.criterion = CRIT_INITIAL_RESIDUAL
    p.max_cg_iters = 0
    p.inner_tol = 1e-3
    p.max_refinements = 60
    for k, v in kw.items():
        if not hasattr(p, k):
            raise AttributeError("unknown mps_params field %r" % k)
        setattr(p, k, v)
    return p


def params_dict(p: MpsParams) -> dict:
    return {name: getattr(p, name) for name, _ in MpsParams._fields_ if not name.startswith("reserved")}
