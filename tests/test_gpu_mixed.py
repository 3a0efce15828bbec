"""Mixed precision: the FP32 operator (the FP64 element matrices rounded to
FP32, or DR terms and element matrices recomputed in FP32) against the FP64
oracle, and FP64 iterative refinement around FP32 inner solves reaching the
FP64 tolerance, with its error against the FP64 oracle solution reported and
bounded."""
import numpy as np
import pytest

from helpers import kat_problem, rel_l2

pytestmark = pytest.mark.gpu

FP32_APPLY_TOL = 2e-5  # FP32 recompute: ~1e-6 typical, bound with margin


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


def fp32_cases(vdr):
    P = vdr.problems
    return {"rotation_VF_64": P.rotation_shear(64, 64, 32, seed=31),
            "const_adv_OT": P.constant_advection(16, 16, 8, seed=32),
            "kat_VF_robin": kat_problem(vdr)}


@pytest.mark.parametrize("name", ["rotation_VF_64", "const_adv_OT",
                                  "kat_VF_robin"])
@pytest.mark.parametrize("mode,op", [("stored", "rounded"),
                                     ("stored", "recompute"),
                                     ("matrix_free", "recompute")])
def test_fp32_operator_against_fp64_oracle(vdr, oracle, gpu_lib, torch, name,
                                           mode, op):
    prob = fp32_cases(vdr)[name]
    m = prob.mesh
    aH, aM = 2.0, 0.7
    bb, _, _ = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                               prob.lam, prob.pdec, prob.q, kod=m.kod,
                               robin_alpha=prob.robin_alpha, aH=aH, aM=aM,
                               want_b=False, want_diag=False, nthreads=8)
    x = np.random.default_rng(8).standard_normal(m.nnode)
    with vdr.Solver(prob, vdr.Options(apply_mode=mode), aH=aH, aM=aM) as s:
        s.set_mixed_operator(op)
        dx = torch.tensor(x, device="cuda")
        dy = torch.empty_like(dx)
        torch.cuda.synchronize()
        for tr in (False, True):
            s.apply32_device(dx, dy, transpose=tr)
            torch.cuda.synchronize()
            yref, _ = oracle.matvec0(m.iss, bb, prob.bc, x, transpose=tr)
            err = rel_l2(dy.cpu().numpy(), yref)
            assert err < FP32_APPLY_TOL, (name, mode, tr, err)
            assert err > 1e-12  # really computed in FP32


HALF_APPLY_TOL = 2e-3  # binary16 rows: <= 2^-11 of each element's largest entry


def half_cases(vdr):
    P = vdr.problems
    return {"rotation_VF_64": (P.rotation_shear(64, 64, 32, seed=31), "atomic"),
            "rotation_VF_64_color": (P.rotation_shear(64, 64, 32, seed=31), "color"),
            "const_adv_OT": (P.constant_advection(16, 16, 8, seed=32), "atomic"),
            "kat_VF_robin": (kat_problem(vdr), "atomic"),
            "two_meshes": (P.concat([P.rotation_cube(6, 41), P.rotation_cube(5, 42)]),
                           "atomic"),
            "ragged_9x7x5": (P.rotation_shear(9, 7, 5, seed=43), "atomic")}


@pytest.mark.parametrize("name", ["rotation_VF_64", "rotation_VF_64_color",
                                  "const_adv_OT", "kat_VF_robin", "two_meshes",
                                  "ragged_9x7x5"])
def test_half_operator_against_fp64_oracle(vdr, oracle, gpu_lib, torch, name):
    """The binary16 inner operator A^ = P A P D^-1 against the oracle's FP64
    element matrices and Jacobi diagonal: structured numbering (warp-
    aggregated scatter), colour order and a connectivity table (two meshes
    in one handle)."""
    prob, scatter = half_cases(vdr)[name]
    m = prob.mesh
    aH, aM = 2.0, 0.7
    bb, _, d = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                               prob.lam, prob.pdec, prob.q, kod=m.kod,
                               robin_alpha=prob.robin_alpha, aH=aH, aM=aM,
                               want_b=False, nthreads=8)
    d[prob.bc == 1] = 1.0
    x = np.random.default_rng(9).standard_normal(m.nnode)
    yref, _ = oracle.matvec0(m.iss, bb, prob.bc, x / d)
    with vdr.Solver(prob, vdr.Options(scatter=scatter), aH=aH, aM=aM) as s:
        s.set_mixed_operator("half")
        dx = torch.tensor(x, dtype=torch.float32, device="cuda")
        dy = torch.empty_like(dx)
        torch.cuda.synchronize()
        s.apply_half_device(dx, dy)
        torch.cuda.synchronize()
        y = dy.cpu().numpy().astype(np.float64)
    err = rel_l2(y, yref)
    assert err < HALF_APPLY_TOL, (name, err)
    assert err > 1e-6  # really rounded to 16 bits
    assert np.all(y[prob.bc == 1] == 0.0)


@pytest.mark.parametrize("solver,op,mode,scatter", [
    ("bicgstab", "rounded", "stored", "atomic"),    # FP32-vector inner solves
    ("bicgstab", "rounded", "stored", "color"),
    ("bicgstab", "half", "stored", "atomic"),       # binary16 inner operator
    ("bicgstab", "half", "stored", "color"),
    ("bicgstab", "recompute", "stored", "atomic"),
    ("bicg", "rounded", "stored", "atomic"),        # FP64-vector inner solves
    ("bicgstab", "recompute", "matrix_free", "atomic")])
def test_mixed_refinement_reaches_fp64_tolerance(vdr, gpu_lib, torch, solver,
                                                 op, mode, scatter):
    prob = vdr.problems.rotation_shear(32, 32, 16, seed=33)
    dt = 10.0 / 32
    aH, aM = 2.0, 3.0 / dt
    opts = vdr.Options(solver=solver, apply_mode=mode, scatter=scatter)
    with vdr.Solver(prob, opts, aH=aH, aM=aM) as s:
        s.set_mixed_operator(op)
        b = torch.empty(prob.mesh.nnode, dtype=torch.float64, device="cuda")
        s.assemble_rhs_device(b, 3.0, 3.0 / dt, None)
        x64 = torch.zeros_like(b)
        it, err64, st = s.solve_device(b, x64, tol=1e-12, itmax=5000)
        assert st == 0
        xm = torch.zeros_like(b)
        torch.cuda.synchronize()
        outer, inner, err, st = s.solve_mixed_device(b, xm, tol=1e-10,
                                                     inner_tol=1e-5)
        torch.cuda.synchronize()
        assert st == 0, (outer, inner, err)
        assert err <= 1e-10
        # BiCG's recurrence residual in the FP32-operator inner solves drifts
        # from the true one, so its correction count varies more
        # (the binary16 operator's rounding takes one or two more corrections)
        assert 1 <= outer <= (4 if solver == "bicgstab" and op != "half" else 6), \
            (outer, inner, err)
        true_rel = s.true_residual_device(b, xm)
        assert true_rel <= 1.5e-10
        # error against the FP64 solution (itself within 1e-12 of the oracle
        # system): bounded by the residual times the conditioning seen here
        assert rel_l2(xm.cpu().numpy(), x64.cpu().numpy()) < 1e-8


@pytest.mark.parametrize("op", ["rounded", "half"])
def test_precision_option_solve_and_time_loop(vdr, gpu_lib, torch, op):
    """Options(precision="mixed") makes vdr_solve and vdr_time_steps run the
    FP64 refinement around FP32 inner solves (FP32 or binary16 inner
    operator): the same FP64 true-residual criterion, the same trajectory as
    the FP64 path to the solve tolerance."""
    prob = vdr.problems.rotation_shear(24, 20, 16, seed=35)
    dt = 10.0 / 24
    aH, aM, cf, rM = 2.0, 3.0 / dt, 3.0, 3.0 / dt
    tol = 1e-11
    out = {}
    for precision in ("fp64", "mixed"):
        opts = vdr.Options(precision=precision)
        with vdr.Solver(prob, opts, aH=aH, aM=aM) as s:
            s.set_mixed_operator(op)
            b = s.assemble_rhs(cf, 0.0, None)
            x, it, err, st = s.solve(b, tol=tol, itmax=5000)
            assert st == 0 and err <= tol, (precision, it, err)
            bd = torch.as_tensor(b, device="cuda")
            xd = torch.as_tensor(x, device="cuda")
            torch.cuda.synchronize()
            assert s.true_residual_device(bd, xd) <= 1.5 * tol
            t = torch.zeros(prob.mesh.nnode, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            masses, its, errs, st, done = s.time_steps_device(t, 4, cf, rM, tol=tol,
                                                              itmax=5000)
            torch.cuda.synchronize()
            assert st == 0 and done == 4 and np.all(errs <= tol), (precision, errs)
            out[precision] = (x, t.cpu().numpy(), masses)
    assert rel_l2(out["mixed"][0], out["fp64"][0]) < 1e-8
    assert rel_l2(out["mixed"][1], out["fp64"][1]) < 1e-8
    assert np.max(np.abs(out["mixed"][2] - out["fp64"][2]) /
                  np.abs(out["fp64"][2])) < 1e-8


def test_fused_inner_barrier_times_out_and_recovers(vdr, gpu_lib, torch):
    """The grid barrier of the fused inner vector kernels (binary16 operator)
    is bounded: a cooperative launch whose second block never arrives makes
    the waiting block give up after its ~1 ms budget, VDR_TIMEOUT reaches the
    host, and a mixed solve on the same handle afterwards (through the fused
    kernels) still reaches its FP64 tolerance."""
    import importlib
    L = importlib.import_module(vdr.__name__ + "._lib")
    prob = vdr.problems.rotation_shear(32, 32, 16, seed=35)
    dt = 10.0 / 32
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=2.0, aM=3.0 / dt) as s:
        assert s.lib.vdr_diag_barrier_timeout(s.h) == L.TIMEOUT
        s.set_mixed_operator("half")
        b = torch.empty(prob.mesh.nnode, dtype=torch.float64, device="cuda")
        s.assemble_rhs_device(b, 3.0, 3.0 / dt, None)
        x = torch.zeros_like(b)
        torch.cuda.synchronize()
        outer, inner, err, st = s.solve_mixed_device(b, x, tol=1e-10, inner_tol=1e-3)
        torch.cuda.synchronize()
        assert st == 0 and err <= 1e-10, (outer, inner, err, st)
        assert s.true_residual_device(b, x) <= 1.5e-10
