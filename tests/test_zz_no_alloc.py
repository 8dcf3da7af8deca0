"""The allocation-free PPE solve (mps_cg_solve_csr_device_noalloc).

Callers that cannot allocate device memory -- an application whose device memory is
reserved by its own caching allocator, or code on a path where cudaMalloc would
synchronize the device -- pass a CSR system already in their device buffers; the
solve keeps its scratch in one fixed static device array.  This test calls it through
the C ABI twice in a row on the same PPE system and checks both results against the
oracle's FP64 CG and the existing entry point (mps_cg_solve_csr), and that the calls
leave free device memory unchanged.  The file name sorts last so that a run stopping
at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from openmps_gb300 import _abi as abi

pytestmark = pytest.mark.gpu

TOL = 1e-9  # relative to max |x|; every side solves to eps = 1e-12


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


def _call(lib, n, d_rp, d_col, d_val, d_b, d_x, eps=1e-12):
    it = C.c_int32()
    rel = C.c_double()
    rc = lib.mps_cg_solve_csr_device_noalloc(
        n, d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr(), d_b.data_ptr(), d_x.data_ptr(),
        eps, abi.CRIT_INITIAL_RESIDUAL, 0, None, C.byref(it), C.byref(rel))
    return rc, it.value, rel.value


def test_noalloc_matches_existing_entry_twice(gpu_lib, oracle_lib):
    torch = pytest.importorskip("torch")
    from oracle.oracle import cg_solve_csr
    from openmps_gb300.computer import Computer

    rp, col, val, b, x0 = _ppe_system()
    n = len(b)
    ora, it_ora, _, _, rc_ora = cg_solve_csr(rp, col, val, b, x0, 1e-12)
    assert rc_ora == 0
    ref, it_ref, _ = Computer(abi.make_params()).cg_solve_csr(rp, col, val, b, x0, 1e-12)

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    d_rp = torch.from_numpy(rp.astype(np.int64)).to(dev)
    d_col = torch.from_numpy(col.astype(np.int32)).to(dev)
    d_val = torch.from_numpy(val.astype(np.float64)).to(dev)
    d_b = torch.from_numpy(b.astype(np.float64)).to(dev)
    d_x0 = torch.from_numpy(x0.astype(np.float64)).to(dev)
    d_x = torch.empty_like(d_x0)
    # warm-up call: the first call in a context may load the library's module, which
    # holds the static scratch array; the calls checked below must change nothing
    d_x.copy_(d_x0)
    rc, _, _ = _call(gpu_lib, n, d_rp, d_col, d_val, d_b, d_x)
    assert rc == abi.MPS_OK, gpu_lib.mps_status_string(rc)
    torch.cuda.synchronize()
    free = [torch.cuda.mem_get_info(dev)[0]]

    for call in range(2):
        d_x.copy_(d_x0)
        rc, it, rel = _call(gpu_lib, n, d_rp, d_col, d_val, d_b, d_x)
        assert rc == abi.MPS_OK, gpu_lib.mps_status_string(rc)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info(dev)[0])
        x = d_x.cpu().numpy()
        err_ora = float(np.max(np.abs(x - ora)) / np.max(np.abs(ora)))
        err_ref = float(np.max(np.abs(x - ref)) / np.max(np.abs(ref)))
        print("call %d: %d iterations (oracle %d, mps_cg_solve_csr %d), rel err vs oracle %.2e, "
              "vs mps_cg_solve_csr %.2e, true relres %.2e" % (call, it, it_ora, it_ref, err_ora,
                                                              err_ref, rel))
        assert err_ora <= TOL, "call %d: rel err vs oracle %.3e" % (call, err_ora)
        assert err_ref <= TOL, "call %d: rel err vs mps_cg_solve_csr %.3e" % (call, err_ref)
        assert abs(it - it_ora) <= max(3, it_ora // 20)
        assert rel < 1e-9
    assert free[0] == free[1] == free[2], "free device memory changed: %s" % free


def test_noalloc_rejects_bad_arguments(gpu_lib):
    n = abi.NOALLOC_MAX_ROWS + 1
    rc = gpu_lib.mps_cg_solve_csr_device_noalloc(n, 1, 1, 1, 1, 1, 1e-8, abi.CRIT_RHS, 0, None, None,
                                                 None)
    assert rc == abi.MPS_ERR_NOALLOC_TOO_LARGE
    # a NULL column or value array is refused on the host, before any launch
    for ptrs in ((1, None, 1, 1, 1), (1, 1, None, 1, 1), (None, 1, 1, 1, 1), (1, 1, 1, None, 1),
                 (1, 1, 1, 1, None)):
        rc = gpu_lib.mps_cg_solve_csr_device_noalloc(16, *ptrs, 1e-8, abi.CRIT_RHS, 0, None, None,
                                                     None)
        assert rc == abi.MPS_ERR_INVALID_ARGUMENT, ptrs
