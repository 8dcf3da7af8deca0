"""The C-ABI library without a GPU: it builds, loads, and exports every symbol that
include/mps.h declares, with struct layouts matching the ctypes mirror."""
import ctypes
import os
import re
import subprocess

import pytest

from openmps_gb300 import _abi as abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "mps.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mps_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(gpu_lib):
    from openmps_gb300 import computer

    names = _declared()
    assert len(names) >= 40
    for name in names:
        assert hasattr(gpu_lib, name), name
    # the ctypes mirror covers the same set
    assert sorted(computer.PROTOTYPES) == names


def test_dynamic_symbol_table(gpu_lib):
    from openmps_gb300 import computer

    out = subprocess.run(["nm", "-D", "--defined-only", computer.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (mps_[a-z0-9_]+)", out))
    assert set(_declared()) <= exported


def test_struct_layouts(gpu_lib):
    assert gpu_lib.mps_params_size() == ctypes.sizeof(abi.MpsParams)
    assert gpu_lib.mps_stats_size() == ctypes.sizeof(abi.MpsStats)
    assert gpu_lib.mps_environment_size() == ctypes.sizeof(abi.MpsEnvironment)


def test_default_params_and_strings(gpu_lib):
    p = abi.MpsParams()
    gpu_lib.mps_default_params(ctypes.byref(p))
    assert p.flags == abi.PRESET_REFERENCE and p.l0 == 0.008 and p.re_by_l0 == 2.4
    assert p.eps == 1e-10 and p.solver == abi.SOLVER_CG64
    assert gpu_lib.mps_status_string(abi.MPS_ERR_CELL_OVERFLOW) == b"too many particles in a cell"
    assert b"sm_103a" in gpu_lib.mps_version()


def test_null_arguments_are_rejected(gpu_lib):
    assert gpu_lib.mps_create(None, 0, None) == abi.MPS_ERR_INVALID_ARGUMENT
    assert gpu_lib.mps_destroy(None) == abi.MPS_ERR_INVALID_ARGUMENT
    assert gpu_lib.mps_forward_time(None, 1e-3) == abi.MPS_ERR_INVALID_ARGUMENT
    assert gpu_lib.mps_particle_count(None) == -1


def test_no_gpu_create_fails_cleanly(gpu_lib):
    # without a device the handle cannot be created; the call reports a CUDA error
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    p = abi.make_params()
    rc = gpu_lib.mps_create(ctypes.byref(p), 0, ctypes.byref(h))
    assert rc == abi.MPS_ERR_CUDA and not h.value
