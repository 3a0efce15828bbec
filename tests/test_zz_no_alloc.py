"""The no-allocation solve entry point (vdr_bicg_noalloc_device), for
callers that cannot allocate device memory, checked through the C ABI
against the drop-in kernel_dbcg_simple_ on two consecutive time steps of
the reference's recorded 7x20x20 case.  Collected last on purpose."""
import ctypes

import numpy as np
import pytest

from helpers import kat_problem, load_kat, rel_l2

pytestmark = pytest.mark.gpu


def test_noalloc_matches_kernel_dbcg_simple_two_calls(vdr, oracle, gpu_lib):
    torch = pytest.importorskip("torch")
    k = load_kat()
    prob = kat_problem(vdr)
    m = prob.mesh
    dt = float(k["dt"])
    tol, itmax = 1e-12, 5000
    t = np.zeros(m.nnode)
    ptr = lambda a: ctypes.c_void_p(int(a.data_ptr()))
    for call in range(2):
        bb, b, diag = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss,
                                      prob.vel, prob.lam, prob.pdec, prob.q,
                                      kod=m.kod, robin_alpha=prob.robin_alpha,
                                      aH=2.0, aM=3.0 / dt, cf=3.0,
                                      rM=3.0 / dt, t_old=t)
        bc = prob.bc
        b[bc == 1] = 0.0
        diag[bc == 1] = 1.0
        t[bc == 1] = 0.0
        x_ref, it_ref, err_ref = vdr.kernel_dbcg_simple(
            m.nnode, b, t, tol, itmax, bb, m.iss, diag, m.nax, m.nay, m.naz, bc)
        d = {name: torch.tensor(arr, device="cuda") for name, arr in
             (("b", b), ("x", t), ("bb", bb), ("diag", diag))}
        d["iss"] = torch.tensor(m.iss.astype(np.int32), device="cuda")
        d["bc"] = torch.tensor(bc.astype(np.int32), device="cuda")
        torch.cuda.synchronize()
        it, err = ctypes.c_int(-1), ctypes.c_double(-1.0)
        st = gpu_lib.vdr_bicg_noalloc_device(
            m.nnode, m.nax, m.nay, m.naz, ptr(d["b"]), ptr(d["x"]), tol, itmax,
            ptr(d["bb"]), ptr(d["iss"]), ptr(d["diag"]), ptr(d["bc"]), None,
            ctypes.byref(it), ctypes.byref(err))
        torch.cuda.synchronize()
        assert st == 0, (call, st, it.value, err.value, it_ref, err_ref)
        x = d["x"].cpu().numpy()
        assert err.value <= tol and err_ref <= tol
        assert rel_l2(x, x_ref) < 1e-9, (call, rel_l2(x, x_ref))
        assert abs(it.value - it_ref) <= 3, (it.value, it_ref)
        t = x_ref


def test_noalloc_rejects_oversized_mesh(vdr, gpu_lib):
    it, err = ctypes.c_int(), ctypes.c_double()
    n = 70 * 70 * 70  # above VDR_NOALLOC_MAX_NODES; no pointer is touched
    st = gpu_lib.vdr_bicg_noalloc_device(
        n, 70, 70, 70, None, None, 1e-8, 10, None, None, None, None, None,
        ctypes.byref(it), ctypes.byref(err))
    assert st == 4
    assert "VDR_NOALLOC_MAX_NODES" in vdr.last_error()
