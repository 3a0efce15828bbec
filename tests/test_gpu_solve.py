"""GPU solve parity through the C ABI: BiCGStab and BiCG solutions against
the oracle (1e-9 relative L2 when both converge tightly), the reference's
recorded 20-step run through both the handle API and the drop-in
kernel_dbcg_simple_, and the solver's edge cases."""
import numpy as np
import pytest

from helpers import kat_problem, load_kat, rel_l2, run_kat_oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def systems(vdr, oracle):
    from oracle.system import reference_system
    P = vdr.problems
    out = {}
    for name, prob in (("const_adv_OT", P.constant_advection(16, 16, 8, seed=21)),
                       ("rotation_VF", P.rotation_shear(16, 16, 8, seed=22))):
        out[name] = (prob, reference_system(prob, tol=1e-13))
    return out


@pytest.mark.parametrize("name", ["const_adv_OT", "rotation_VF"])
@pytest.mark.parametrize("solver", ["bicgstab", "bicg"])
@pytest.mark.parametrize("mode,scatter,store", [("stored", "atomic", "df"),
                                                ("stored", "color", "df"),
                                                ("stored", "warp", "df"),
                                                ("stored", "atomic", "fp64"),
                                                ("matrix_free", "atomic", "auto")])
def test_solution_parity(vdr, gpu_lib, systems, name, solver, mode, scatter,
                         store):
    prob, ref = systems[name]
    assert ref["status"] == 0
    opts = vdr.Options(solver=solver, apply_mode=mode, scatter=scatter,
                       matrix_storage=store)
    with vdr.Solver(prob, opts) as s:
        x, it, err, st = s.solve(ref["b"], tol=1e-13, itmax=20000)
    assert st == 0, (st, it, err)
    assert err <= 1e-13
    assert rel_l2(x, ref["x_solution"]) < 1e-9


@pytest.mark.parametrize("solver", ["bicgstab", "bicg"])
def test_iteration_count_matches_oracle(vdr, oracle, gpu_lib, systems, solver):
    """Away from the rounding floor (tol 1e-10) the GPU and the oracle take
    the same number of iterations up to a few (reductions sum in a
    different order)."""
    prob, ref = systems["const_adv_OT"]
    m = prob.mesh
    fn = oracle.bicgstab if solver == "bicgstab" else oracle.dbcg
    _, it_ref, _, st_ref = fn(ref["b"], np.zeros(m.nnode), ref["bb"], m.iss,
                              ref["diag"], prob.bc, 1e-10, 20000)
    assert st_ref == 0
    with vdr.Solver(prob, vdr.Options(solver=solver)) as s:
        _, it, _, st = s.solve(ref["b"], tol=1e-10, itmax=20000)
    assert st == 0
    assert abs(it - it_ref) <= max(3, 0.1 * it_ref), (it, it_ref)


def test_kat_run_handle_api(vdr, oracle, gpu_lib):
    """The recorded 7x20x20, 20-step run with assembly on the GPU
    (vdr_assemble_rhs) and BiCG on the GPU."""
    k = load_kat()
    prob = kat_problem(vdr)
    dt = float(k["dt"])
    m = prob.mesh
    t = np.zeros(m.nnode)
    its, masses = [], []
    with vdr.Solver(prob, vdr.Options(solver="bicg"), aH=2.0, aM=3.0 / dt) as s:
        for step in range(k["steps"]):
            b = s.assemble_rhs(3.0, 3.0 / dt, t)
            t, it, err, st = s.solve(b, t, tol=k["tol"], itmax=k["itmax"])
            assert st == 0
            its.append(it)
            masses.append(s.mass(t))
    ref_its = k["log"]["iterations"]
    assert all(abs(a - b) <= 2 for a, b in zip(its, ref_its)), its
    ref_m = np.array(k["log"]["masses"])
    assert np.max(np.abs(np.array(masses) - ref_m) / ref_m) < 1e-6


def test_kat_run_dropin_kernel_dbcg_simple(vdr, oracle, gpu_lib):
    """Same run through the reference's own entry point with the oracle's
    host-assembled BB, exactly as VANADIS.FOR:793-810 calls it."""
    k = load_kat()
    prob = kat_problem(vdr)
    m = prob.mesh
    dt = float(k["dt"])
    t = np.zeros(m.nnode)
    its, masses = [], []
    for step in range(k["steps"]):
        bb, b, diag = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss,
                                      prob.vel, prob.lam, prob.pdec, prob.q,
                                      kod=m.kod, robin_alpha=prob.robin_alpha,
                                      aH=2.0, aM=3.0 / dt, cf=3.0,
                                      rM=3.0 / dt, t_old=t)
        bc = prob.bc
        b[bc == 1] = 0.0
        diag[bc == 1] = 1.0
        t[bc == 1] = 0.0
        t, it, err = vdr.kernel_dbcg_simple(m.nnode, b, t, k["tol"], k["itmax"],
                                            bb, m.iss, diag, m.nax, m.nay,
                                            m.naz, bc)
        assert err <= k["tol"]
        its.append(it)
        masses.append(oracle.integrate_mass(m.iss, m.xx, m.yy, m.zz, t))
    assert all(abs(a - b) <= 2 for a, b in zip(its, k["log"]["iterations"])), its
    ref_m = np.array(k["log"]["masses"])
    assert np.max(np.abs(np.array(masses) - ref_m) / ref_m) < 1e-6


def test_dropin_matches_oracle_dbcg(vdr, oracle, gpu_lib):
    """The drop-in's BiCG against the oracle's on the same BB.  The drop-in
    holds BB as double-float pairs (2^-48 relative), so at tol 1e-13 the
    iteration count may differ from the oracle's FP64 BiCG by a few; the
    solution agrees to 1e-9."""
    prob = kat_problem(vdr)
    m = prob.mesh
    bb, b, diag = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss,
                                  prob.vel, prob.lam, prob.pdec, prob.q,
                                  kod=m.kod, robin_alpha=prob.robin_alpha,
                                  aH=2.0, aM=0.03, cf=3.0, rM=0.03)
    b[prob.bc == 1] = 0.0
    diag[prob.bc == 1] = 1.0
    x0 = np.zeros(m.nnode)
    xr, itr, er, _ = oracle.dbcg(b, x0, bb, m.iss, diag, prob.bc, 1e-13, 5000)
    x, it, err = vdr.kernel_dbcg_simple(m.nnode, b, x0, 1e-13, 5000, bb, m.iss,
                                        diag, m.nax, m.nay, m.naz, prob.bc)
    assert err <= 1e-13
    assert rel_l2(x, xr) < 1e-9
    assert abs(it - itr) <= 6


def test_dropin_store_window_fallback(vdr, oracle, gpu_lib):
    """BB entries beyond the double-float store's window (the system scaled
    by 1e40, which leaves the solution unchanged) put the drop-in on the
    FP64 store; the next call with ordinary entries goes back to the pair
    store.  Every call agrees with the oracle's BiCG."""
    prob = kat_problem(vdr)
    m = prob.mesh
    bb, b, diag = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss,
                                  prob.vel, prob.lam, prob.pdec, prob.q,
                                  kod=m.kod, robin_alpha=prob.robin_alpha,
                                  aH=2.0, aM=0.03, cf=3.0, rM=0.03)
    b[prob.bc == 1] = 0.0
    diag[prob.bc == 1] = 1.0
    x0 = np.zeros(m.nnode)
    xr, _, _, _ = oracle.dbcg(b, x0, bb, m.iss, diag, prob.bc, 1e-13, 5000)
    for scale in (1.0, 1e40, 1.0):
        x, it, err = vdr.kernel_dbcg_simple(m.nnode, b * scale, x0.copy(), 1e-13,
                                            5000, bb * scale, m.iss,
                                            diag * scale, m.nax, m.nay, m.naz,
                                            prob.bc)
        assert err <= 1e-13, scale
        assert rel_l2(x, xr) < 1e-9, scale


@pytest.mark.parametrize("scatter,store", [("atomic", "df"), ("color", "df"),
                                           ("atomic", "fp64")])
def test_element_matrices_export_round_trip(vdr, oracle, gpu_lib, scatter,
                                            store):
    """vdr_get_element_matrices returns the GPU-built operator in the
    reference's BB layout and element order (the colour scatter stores
    elements permuted): it matches the oracle's BB, and fed back to
    kernel_dbcg_simple it gives the oracle's BiCG solution."""
    prob = kat_problem(vdr)
    m = prob.mesh
    aH, aM = 2.0, 0.03
    bb, b, diag = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss,
                                  prob.vel, prob.lam, prob.pdec, prob.q,
                                  kod=m.kod, robin_alpha=prob.robin_alpha,
                                  aH=aH, aM=aM, cf=3.0, rM=aM)
    b[prob.bc == 1] = 0.0
    diag[prob.bc == 1] = 1.0
    opts = vdr.Options(scatter=scatter, matrix_storage=store)
    with vdr.Solver(prob, opts, aH=aH, aM=aM) as s:
        bbg = s.element_matrices()
        dg = s.diag()
    assert rel_l2(bbg, bb) < 1e-12
    assert rel_l2(dg, diag) < 1e-12
    x0 = np.zeros(m.nnode)
    xr, _, _, _ = oracle.dbcg(b, x0, bb, m.iss, diag, prob.bc, 1e-13, 5000)
    x, it, err = vdr.kernel_dbcg_simple(m.nnode, b, x0.copy(), 1e-13, 5000, bbg,
                                        m.iss, dg, m.nax, m.nay, m.naz, prob.bc)
    assert err <= 1e-13
    assert rel_l2(x, xr) < 1e-9


def test_zero_rhs_gives_zero(vdr, gpu_lib):
    prob = vdr.problems.rotation_shear(6, 6, 4, seed=3)
    with vdr.Solver(prob) as s:
        x, it, err, st = s.solve(np.zeros(prob.mesh.nnode),
                                 np.ones(prob.mesh.nnode))
    assert st == 0 and it == 0 and np.all(x == 0.0)


def test_converged_initial_guess_takes_no_iteration(vdr, gpu_lib, systems):
    prob, ref = systems["rotation_VF"]
    with vdr.Solver(prob) as s:
        x, it, err, st = s.solve(ref["b"], ref["x_solution"], tol=1e-8)
    assert st == 0 and it == 0 and err <= 1e-8


def test_itmax_reports_not_converged(vdr, gpu_lib, systems):
    prob, ref = systems["rotation_VF"]
    for solver in ("bicgstab", "bicg"):
        with vdr.Solver(prob, vdr.Options(solver=solver)) as s:
            x, it, err, st = s.solve(ref["b"], tol=1e-14, itmax=5)
        assert st == 1 and it == 5 and err > 1e-14


def test_dirichlet_entries_of_solution_are_zero(vdr, gpu_lib, systems):
    prob, ref = systems["const_adv_OT"]
    x0 = np.random.default_rng(9).standard_normal(prob.mesh.nnode)
    with vdr.Solver(prob) as s:
        x, it, err, st = s.solve(ref["b"], x0, tol=1e-10)
    assert st == 0 and np.all(x[prob.bc == 1] == 0.0)


def test_true_residual_device(vdr, gpu_lib, systems):
    torch = pytest.importorskip("torch")
    prob, ref = systems["rotation_VF"]
    with vdr.Solver(prob) as s:
        b = torch.tensor(ref["b"], device="cuda")
        x = torch.zeros_like(b)
        torch.cuda.synchronize()  # the handle runs on its own stream
        it, err, st = s.solve_device(b, x, tol=1e-10)
        torch.cuda.synchronize()
        rel = s.true_residual_device(b, x)
    assert st == 0 and rel < 1e-9


def test_kat_run_device_time_loop(vdr, gpu_lib):
    """The recorded 20-step run in one call of the device-resident time loop
    (assembly, solve and mass integral on the GPU)."""
    torch = pytest.importorskip("torch")
    k = load_kat()
    prob = kat_problem(vdr)
    dt = float(k["dt"])
    with vdr.Solver(prob, vdr.Options(solver="bicg"), aH=2.0, aM=3.0 / dt) as s:
        t = torch.zeros(prob.mesh.nnode, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        masses, its, errs, st, done = s.time_steps_device(
            t, k["steps"], 3.0, 3.0 / dt, tol=k["tol"], itmax=k["itmax"])
    assert st == 0 and done == k["steps"]
    assert all(abs(a - b) <= 2 for a, b in zip(its, k["log"]["iterations"])), its
    ref_m = np.array(k["log"]["masses"])
    assert np.max(np.abs(masses - ref_m) / ref_m) < 1e-6
    assert np.all(errs <= k["tol"])


@pytest.mark.parametrize("scatter,store", [("atomic", "df"), ("color", "df"),
                                           ("atomic", "fp64")])
def test_time_loop_stored_mass_matches_step_by_step(vdr, gpu_lib, scatter, store):
    """From its second step the device time loop forms the right-hand side
    from the stored A and M (b = cf F - (A T)/aH + (aM/aH + rM) M T); the
    trajectory equals a step-by-step loop whose every right-hand side is a
    full Gauss pass (vdr_assemble_rhs), to the solve tolerance."""
    import torch
    prob = vdr.problems.rotation_shear(12, 10, 8, seed=71)
    prob.pdec[:] = 0.2
    prob.robin_alpha = 0.4
    dt = 10.0 / 12
    aH, aM, cf, rM = 2.0, 3.0 / dt, 3.0, 3.0 / dt
    steps, tol = 5, 1e-12
    opts = vdr.Options(scatter=scatter, matrix_storage=store)
    with vdr.Solver(prob, opts, aH=aH, aM=aM) as s:
        t = torch.zeros(prob.mesh.nnode, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        masses, its, errs, st, done = s.time_steps_device(t, steps, cf, rM, tol=tol,
                                                          itmax=5000)
        torch.cuda.synchronize()
        assert st == 0 and done == steps
        t_loop = t.cpu().numpy()
    with vdr.Solver(prob, opts, aH=aH, aM=aM) as s:
        th = np.zeros(prob.mesh.nnode)
        m_ref = []
        for k in range(steps):
            b = s.assemble_rhs(cf, rM, th)
            th, it, err, st = s.solve(b, th, tol=tol, itmax=5000)
            assert st == 0
            m_ref.append(s.mass(th))
    assert rel_l2(t_loop, th) < 1e-9
    assert np.max(np.abs(masses - np.array(m_ref)) / np.abs(np.array(m_ref))) < 1e-9


@pytest.mark.parametrize("restart", [1, 5, 20])
def test_gcr_jacobi_matches_bicgstab(vdr, oracle, gpu_lib, restart):
    """Restarted GCR with Jacobi (the flexible solver of the learned path)
    reaches the tolerance and the same solution as BiCGStab; its residual
    never increases (the reported residual is the true FP64 residual)."""
    import torch
    prob = vdr.problems.rotation_shear(9, 8, 6, seed=61)
    aH, aM = 2.0, 3.0 / (10.0 / 9)
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        b = torch.as_tensor(s.assemble_rhs(3.0, 0.0, None), device="cuda")
        x1 = torch.zeros_like(b)
        x2 = torch.zeros_like(b)
        torch.cuda.synchronize()
        it1, e1, st1 = s.solve_device(b, x1, tol=1e-11, itmax=5000)
        it2, e2, st2, fb = s.solve_gcr_device(b, x2, tol=1e-11, itmax=5000,
                                              restart=restart)
        true2 = s.true_residual_device(b, x2)
        torch.cuda.synchronize()
        X1, X2 = x1.cpu().numpy(), x2.cpu().numpy()
    assert st1 == 0 and st2 == 0 and not fb
    assert e2 <= 1e-11 and true2 <= 1.01e-11
    assert rel_l2(X2, X1) < 1e-8
    assert np.all(X2[prob.bc == 1] == 0.0)
