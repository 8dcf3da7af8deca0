"""The allocation-free PPE solve (mps_cg_solve_csr_device_noalloc).

Callers that cannot allocate device memory -- an application whose device memory is
reserved by its own caching allocator, or code on a path where cudaMalloc would
synchronize the device -- pass a CSR system already in their device buffers; the
solve keeps its scratch in one fixed static device array.  This test calls it through
the C ABI twice in a row on the same PPE system and checks both results against the
existing entry point (mps_cg_solve_csr) and that the calls leave free device memory
unchanged.  The file name sorts last so that a run stopping at the first failure has
run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from openmps_gb300 import _abi as abi

pytestmark = pytest.mark.gpu

TOL = 1e-9  # relative to max |x|; both sides solve to eps = 1e-12


def _ppe_system():
    from helpers import stock_tank
    from oracle.oracle import Oracle

    s = stock_tank()
    o = Oracle(s.params())
    o.add_scene(s)
    for _ in range(3):
        o.forward_time(s.meta["dt"])
    o.begin_step(s.meta["dt"])
    for st in ("search_neighbor", "density", "error_correction", "explicit", "density", "save_x",
               "set_ppe"):
        o.stage(st)
    return o.ppe()


def test_noalloc_matches_existing_entry_twice(gpu_lib, oracle_lib):
    torch = pytest.importorskip("torch")
    from openmps_gb300.computer import Computer

    rp, col, val, b, x0 = _ppe_system()
    n = len(b)
    ref, it_ref, _ = Computer(abi.make_params()).cg_solve_csr(rp, col, val, b, x0, 1e-12)

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    d_rp = torch.from_numpy(rp.astype(np.int64)).to(dev)
    d_col = torch.from_numpy(col.astype(np.int32)).to(dev)
    d_val = torch.from_numpy(val.astype(np.float64)).to(dev)
    d_b = torch.from_numpy(b.astype(np.float64)).to(dev)
    torch.cuda.synchronize()

    free_after = []
    for call in range(2):
        d_x = torch.from_numpy(x0.astype(np.float64)).to(dev)
        torch.cuda.synchronize()
        it = C.c_int32()
        rel = C.c_double()
        rc = gpu_lib.mps_cg_solve_csr_device_noalloc(
            n, d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr(), d_b.data_ptr(), d_x.data_ptr(),
            1e-12, abi.CRIT_INITIAL_RESIDUAL, 0, None, C.byref(it), C.byref(rel))
        assert rc == abi.MPS_OK, gpu_lib.mps_status_string(rc)
        x = d_x.cpu().numpy()
        err = float(np.max(np.abs(x - ref)) / np.max(np.abs(ref)))
        assert err <= TOL, "call %d: rel err %.3e" % (call, err)
        assert abs(it.value - it_ref) <= max(3, it_ref // 20)
        assert rel.value < 1e-9
        free_after.append(torch.cuda.mem_get_info(dev)[0])
    assert free_after[0] == free_after[1]


def test_noalloc_rejects_oversized_systems(gpu_lib):
    n = abi.NOALLOC_MAX_ROWS + 1
    rc = gpu_lib.mps_cg_solve_csr_device_noalloc(n, 1, 1, 1, 1, 1, 1e-8, abi.CRIT_RHS, 0, None, None,
                                                 None)
    assert rc == abi.MPS_ERR_NOALLOC_TOO_LARGE
