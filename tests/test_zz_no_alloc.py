"""The no-allocation solve entry point (vdr_bicg_noalloc_device), for
callers that cannot allocate device memory because another allocator or a
fixed budget owns the device after start-up.  Checked through the C ABI on
two consecutive time steps of the reference's recorded 7x20x20 case against
the oracle's BiCG (dbcg_simple, vanadis_full_DR_OpenMP_timing.for:906-984)
and against the drop-in kernel_dbcg_simple_; a right-hand side that is
nonzero on Dirichlet nodes (which the reference keeps in its residual); the
device's free memory unchanged across a call; oversized meshes rejected.
Collected last on purpose: the module runs after every other test."""
import ctypes

import numpy as np
import pytest

from helpers import kat_problem, load_kat, rel_l2

pytestmark = pytest.mark.gpu

VDR_OK, VDR_NOT_CONVERGED, VDR_BAD_ARGUMENT = 0, 1, 4


def _ptr(t):
    return ctypes.c_void_p(int(t.data_ptr()))


class _DeviceInputs:
    """Device copies of one system, allocated once so that the calls under
    test run with no allocation of the test's own in between."""

    def __init__(self, torch, m, bb, iss, bc):
        self.torch = torch
        n = m.nnode
        self.b = torch.zeros(n, dtype=torch.float64, device="cuda")
        self.x = torch.zeros(n, dtype=torch.float64, device="cuda")
        self.diag = torch.zeros(n, dtype=torch.float64, device="cuda")
        self.bb = torch.tensor(bb, device="cuda")
        self.iss = torch.tensor(np.ascontiguousarray(iss, dtype=np.int32),
                                device="cuda")
        self.bc = torch.tensor(np.asarray(bc, dtype=np.int32), device="cuda")
        self.m = m

    def set(self, b, x, diag, bb=None):
        T = self.torch
        self.b.copy_(T.from_numpy(np.ascontiguousarray(b)))
        self.x.copy_(T.from_numpy(np.ascontiguousarray(x)))
        self.diag.copy_(T.from_numpy(np.ascontiguousarray(diag)))
        if bb is not None:
            self.bb.copy_(T.from_numpy(np.ascontiguousarray(bb)))
        T.cuda.synchronize()

    def call(self, lib, tol, itmax):
        m = self.m
        it, err = ctypes.c_int(-1), ctypes.c_double(-1.0)
        st = lib.vdr_bicg_noalloc_device(
            m.nnode, m.nax, m.nay, m.naz, _ptr(self.b), _ptr(self.x), tol,
            itmax, _ptr(self.bb), _ptr(self.iss), _ptr(self.diag),
            _ptr(self.bc), None, ctypes.byref(it), ctypes.byref(err))
        self.torch.cuda.synchronize()
        return st, it.value, err.value, self.x.cpu().numpy()


def _step_system(oracle, prob, dt, t):
    m = prob.mesh
    bb, b, diag = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss,
                                  prob.vel, prob.lam, prob.pdec, prob.q,
                                  kod=m.kod, robin_alpha=prob.robin_alpha,
                                  aH=2.0, aM=3.0 / dt, cf=3.0, rM=3.0 / dt,
                                  t_old=t)
    bc = prob.bc
    b[bc == 1] = 0.0
    diag[bc == 1] = 1.0
    return bb, b, diag


def test_noalloc_two_calls_match_oracle_and_dropin(vdr, oracle, gpu_lib):
    """Two time steps in a row (the second starts from the first's solution,
    the shared scratch keeping the first call's contents): each solution
    against the oracle's BiCG to 1e-9 and its iteration count within 3, and
    against kernel_dbcg_simple_; the device's free memory is the same before
    and after the second call."""
    torch = pytest.importorskip("torch")
    k = load_kat()
    prob = kat_problem(vdr)
    m = prob.mesh
    dt = float(k["dt"])
    tol, itmax = 1e-12, 5000
    t = np.zeros(m.nnode)
    bb, _, _ = _step_system(oracle, prob, dt, t)
    dev = _DeviceInputs(torch, m, bb, m.iss, prob.bc)
    for call in range(2):
        bb, b, diag = _step_system(oracle, prob, dt, t)
        t0 = t.copy()
        t0[prob.bc == 1] = 0.0
        x_or, it_or, err_or, st_or = oracle.dbcg(b, t0, bb, m.iss, diag, prob.bc,
                                                 tol, itmax)
        assert st_or == 0 and err_or <= tol
        x_dr, it_dr, err_dr = vdr.kernel_dbcg_simple(
            m.nnode, b, t0, tol, itmax, bb, m.iss, diag, m.nax, m.nay, m.naz,
            prob.bc)
        dev.set(b, t, diag, bb)
        free_before = torch.cuda.mem_get_info()[0]
        st, it, err, x = dev.call(gpu_lib, tol, itmax)
        free_after = torch.cuda.mem_get_info()[0]
        assert st == VDR_OK, (call, st, it, err, it_or, err_or)
        assert err <= tol
        assert rel_l2(x, x_or) < 1e-9, (call, rel_l2(x, x_or))
        assert abs(it - it_or) <= 3, (call, it, it_or)
        assert rel_l2(x, x_dr) < 1e-9, (call, rel_l2(x, x_dr))
        assert np.all(x[prob.bc == 1] == 0.0)
        if call == 1:   # the first call may load the library's device code
            assert free_after == free_before, (free_before, free_after)
        t = x_or


def test_noalloc_dirichlet_rhs_kept_in_residual(vdr, oracle, gpu_lib):
    """A right-hand side that is nonzero on Dirichlet nodes: as in the
    reference, those entries stay in the residual (its norm cannot fall
    below theirs) and enter the Jacobi inner products.  A fixed number of
    iterations (tolerance below that floor): iteration count, residual and
    iterate against the oracle's BiCG and against kernel_dbcg_simple_."""
    torch = pytest.importorskip("torch")
    k = load_kat()
    prob = kat_problem(vdr)
    m = prob.mesh
    bb, b, diag = _step_system(oracle, prob, float(k["dt"]), np.zeros(m.nnode))
    dmask = prob.bc == 1
    b[dmask] = 1e-3 * np.abs(b).max() * np.cos(np.arange(int(dmask.sum())))
    floor = np.linalg.norm(b[dmask]) / np.linalg.norm(b)
    tol, itmax = 1e-14, 30
    x0 = np.zeros(m.nnode)
    x_or, it_or, err_or, st_or = oracle.dbcg(b, x0, bb, m.iss, diag, prob.bc,
                                             tol, itmax)
    assert st_or == 1 and it_or == itmax and err_or >= floor
    x_dr, it_dr, err_dr = vdr.kernel_dbcg_simple(
        m.nnode, b, x0, tol, itmax, bb, m.iss, diag, m.nax, m.nay, m.naz,
        prob.bc)
    dev = _DeviceInputs(torch, m, bb, m.iss, prob.bc)
    dev.set(b, x0, diag)
    st, it, err, x = dev.call(gpu_lib, tol, itmax)
    assert st == VDR_NOT_CONVERGED and it == itmax == it_dr
    assert err >= floor * (1.0 - 1e-12)
    assert abs(err - err_or) <= 1e-6 * err_or, (err, err_or)
    assert abs(err - err_dr) <= 1e-6 * err_dr, (err, err_dr)
    assert rel_l2(x, x_or) < 1e-8, rel_l2(x, x_or)
    assert rel_l2(x, x_dr) < 1e-8, rel_l2(x, x_dr)


def test_noalloc_rejects_oversized_mesh(vdr, gpu_lib):
    it, err = ctypes.c_int(), ctypes.c_double()
    n = 70 * 70 * 70  # above VDR_NOALLOC_MAX_NODES; no pointer is touched
    st = gpu_lib.vdr_bicg_noalloc_device(
        n, 70, 70, 70, None, None, 1e-8, 10, None, None, None, None, None,
        ctypes.byref(it), ctypes.byref(err))
    assert st == VDR_BAD_ARGUMENT
    assert "VDR_NOALLOC_MAX_NODES" in vdr.last_error()
