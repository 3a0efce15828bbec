"""The element build from the mesh's geometric factors (VDR_BUILD_AUTO: J^-1
and detJ at the Gauss points and the unit-diffusivity stiffness formed once
per handle) against the build that evaluates the Jacobians from the
coordinates every time (VDR_BUILD_RECOMPUTE) and against the oracle:
element matrices, Jacobi diagonal, right-hand side with T_old, the FP64 and
double-float stores, the time loop's M store; the fallback for Robin
elements; the status call.  Bars: 1e-12 relative L2 against the oracle (as
every FP64 operator test), 1e-13 between the two builds (both are
double-float evaluations of the same integrals)."""
import copy

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_MODES = 1e-13


def cases(vdr):
    P = vdr.problems
    out = {
        "const_adv_OT": P.constant_advection(8, 8, 4, seed=21),
        "rotation_VF": P.rotation_shear(9, 7, 5, seed=22),
        "rotation_GP": P.rotation_shear(7, 6, 5, seed=23, variant=P.DR_GP),
        "one_element": P.rotation_shear(1, 1, 1, seed=24),
        "brick_axis": P.uniform_fields_problem(
            "axis", P.axis_mesh(np.linspace(0, 1, 6), np.linspace(0, 0.5, 4) ** 1.5,
                                np.linspace(0, 2, 5)),
            lam=1e-3, pdec=0.0, vel3=(1.0, 0.4, -0.2)),
    }
    out["rotation_GP"].lam[:] = 0.02
    p = P.rotation_shear(5, 4, 6, seed=26)
    p.pdec[:] = 0.3
    out["rotation_decay"] = p
    # VF with the element Peclet number spread over 1e-4 .. 1e4 (diffusivity
    # log-uniform over eight decades): every branch of the double-float
    # beta(Pe) (series, exponential form, 1 - 1/Pe)
    p = P.rotation_shear(8, 7, 6, seed=29)
    p.lam[:] = 10.0 ** np.random.default_rng(30).uniform(-5.0, 3.0, p.lam.size)
    out["vf_peclet_sweep"] = p
    # Robin faces present but a zero Robin coefficient: the cached build
    p = P.rotation_shear(4, 5, 3, seed=27)
    p.robin_alpha = 0.0
    out["robin_faces_alpha0"] = p
    return out


@pytest.fixture(scope="module")
def problems(vdr):
    return cases(vdr)


NAMES = ["const_adv_OT", "rotation_VF", "rotation_GP", "one_element",
         "brick_axis", "rotation_decay", "vf_peclet_sweep", "robin_faces_alpha0"]


def oracle_system(oracle, prob, aH, aM, cf, rM, t_old):
    m = prob.mesh
    bb, b, d = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                               prob.lam, prob.pdec, prob.q, kod=m.kod,
                               robin_alpha=prob.robin_alpha, aH=aH, aM=aM,
                               cf=cf, rM=rM, t_old=t_old)
    b[prob.bc == 1] = 0.0
    d[prob.bc == 1] = 1.0
    return bb, b, d


def build_all(vdr, prob, mode, store, aH, aM, cf, rM, t_old):
    opts = vdr.Options(apply_mode="stored", matrix_storage=store)
    with vdr.Solver(prob, opts, aH=aH, aM=aM) as s:
        s.set_build_mode(mode)
        b = s.assemble_rhs(cf, rM, t_old)   # operator + RHS in one pass
        bb = s.element_matrices()
        d = s.diag()
        b2 = s.assemble_rhs(cf, rM, t_old)  # RHS alone, operator valid
        status = s.geometry_status()
        # a rebuild is four launches (per-element scalars, build, Dirichlet
        # fix of the diagonal, element masks): no redo with FP64 rows (a
        # value outside the pair window, such as a Gaussian source's far
        # tail, must not send the build there)
        s.set_operator(aH, aM)
        n0 = vdr.kernel_launch_count()
        s.assemble_rhs(cf, rM, t_old)
        launches = vdr.kernel_launch_count() - n0
    return bb, b, d, b2, status, launches


@pytest.mark.parametrize("store", ["df", "fp64"])
@pytest.mark.parametrize("name", NAMES)
def test_cached_build_matches_recompute_and_oracle(vdr, oracle, gpu_lib, problems,
                                                   name, store):
    prob = problems[name]
    m = prob.mesh
    dt = 0.05
    aH, aM, cf, rM = 2.0, 3.0 / dt, 3.0, 3.0 / dt
    t_old = np.random.default_rng(31).standard_normal(m.nnode)
    t_old[prob.bc == 1] = 0.0
    bb_ref, b_ref, d_ref = oracle_system(oracle, prob, aH, aM, cf, rM, t_old)
    got = {mode: build_all(vdr, prob, mode, store, aH, aM, cf, rM, t_old)
           for mode in ("auto", "recompute")}
    for mode, (bb, b, d, b2, status, launches) in got.items():
        assert launches == 4, (name, mode, launches)
        assert rel_l2(bb, bb_ref) < TOL, (name, mode)
        assert rel_l2(b, b_ref) < TOL, (name, mode)
        assert rel_l2(b2, b_ref) < TOL, (name, mode)
        assert rel_l2(d, d_ref) < TOL, (name, mode)
    st_auto, nbytes = got["auto"][4]
    assert st_auto == 1 and nbytes == 928 * m.nelem
    assert got["recompute"][4] == (0, 0)
    bb_a, bb_r = got["auto"][0], got["recompute"][0]
    scale = np.abs(bb_r).max()
    # GP's beta(Pe) is coth(Pe) - 1/Pe through exp in FP64 (the variant's
    # own form), which magnifies its input's rounding by ~3/Pe^2 at small Pe:
    # the two builds form Pe with different roundings
    tol = 1e-12 if prob.variant == vdr.problems.DR_GP else TOL_MODES
    assert np.abs(bb_a - bb_r).max() <= tol * scale, name
    assert rel_l2(got["auto"][1], got["recompute"][1]) < tol


def test_robin_term_takes_the_recompute_build(vdr, oracle, gpu_lib):
    P = vdr.problems
    prob = P.rotation_shear(5, 4, 6, seed=28)
    prob.pdec[:] = 0.3
    prob.robin_alpha = 0.7
    aH, aM = 2.0, 0.37
    bb_ref, _, _ = oracle_system(oracle, prob, aH, aM, 1.0, 0.0, None)
    with vdr.Solver(prob, aH=aH, aM=aM) as s:
        bb = s.element_matrices()
        assert s.geometry_status() == (0, 0)
    assert rel_l2(bb, bb_ref) < TOL


def test_fields_change_between_builds(vdr, oracle, gpu_lib, problems):
    """The factors hold geometry only: new velocity, diffusivity and decay
    fields on the same handle give the oracle's operator for the new
    fields."""
    prob = copy.deepcopy(problems["rotation_VF"])
    aH, aM = 2.0, 5.0
    rng = np.random.default_rng(32)
    with vdr.Solver(prob, aH=aH, aM=aM) as s:
        s.element_matrices()
        for k in range(2):
            prob.vel[:] = rng.standard_normal(prob.vel.size) * (0.5 + k)
            prob.lam[:] = np.exp(np.log(1e-3) + rng.standard_normal(prob.lam.size))
            prob.pdec[:] = 0.1 * k
            s.set_fields(prob.vel, prob.lam, prob.pdec, prob.q)
            bb = s.element_matrices()
            bb_ref, _, _ = oracle_system(oracle, prob, aH, aM, 1.0, 0.0, None)
            assert rel_l2(bb, bb_ref) < TOL, k
        assert s.geometry_status()[0] == 1


def test_time_loop_modes_agree(vdr, gpu_lib, problems):
    """vdr_time_steps keeps M and F from its first build (the SPLIT build
    with the M store): three steps from the same T_0 in both modes."""
    import torch
    prob = problems["rotation_decay"]
    dt = 0.05
    cf, rM = 3.0, 3.0 / dt
    t0 = np.random.default_rng(33).random(prob.mesh.nnode)
    out = {}
    for mode in ("auto", "recompute"):
        with vdr.Solver(prob, aH=2.0, aM=3.0 / dt) as s:
            s.set_build_mode(mode)
            t = torch.as_tensor(t0, device="cuda")
            masses, its, errs, st, done = s.time_steps_device(t, 3, cf, rM, tol=1e-12)
            torch.cuda.synchronize()
            assert st == 0 and done == 3, (mode, st, done)
            out[mode] = (t.cpu().numpy(), masses)
    assert rel_l2(out["auto"][0], out["recompute"][0]) < 1e-9
    assert np.allclose(out["auto"][1], out["recompute"][1], rtol=1e-9, atol=0.0)


def test_build_mode_argument_checked(vdr, gpu_lib, problems):
    with vdr.Solver(problems["one_element"]) as s:
        with pytest.raises(KeyError):
            s.set_build_mode("sometimes")
        assert s.lib.vdr_set_build_mode(s.h, 7) == 4  # VDR_BAD_ARGUMENT


def beta_exact(x):
    """coth x - 1/x to ~40 digits (decimal arithmetic)."""
    from decimal import Decimal, getcontext
    getcontext().prec = 60
    d = Decimal(x)
    if d < Decimal("1e-3"):  # series, far below the rounding of the other form
        y = d * d
        return float(d / 3 - d * y / 45 + 2 * d * y * y / 945 - d * y ** 3 / 4725)
    e = (2 * d).exp()
    return float((e + 1) / (e - 1) - 1 / d)


def test_double_float_beta_vf(vdr, gpu_lib):
    """The build's beta(Pe) of the VF variant in double-float against the
    exact function, across its three branches and their boundaries."""
    import ctypes
    xs = np.concatenate([np.logspace(-12, 4, 400),
                         [0.4999999, 0.5, 0.5000001, 43.999, 44.0, 44.001,
                          1e-3, 0.1, 1.0, 3.7, 709.0]])
    got = np.zeros_like(xs)
    lib = vdr.load_library()
    D = ctypes.POINTER(ctypes.c_double)
    st = lib.vdr_diag_beta_vf(int(xs.size), xs.ctypes.data_as(D), got.ctypes.data_as(D))
    assert st == 0
    ref = np.array([beta_exact(x) for x in xs])
    rel = np.abs(got - ref) / np.abs(ref)
    # largest just above 1/2, where 1 - 1/x and 2u/(1 - u) cancel by ~5
    assert rel.max() < 2.5e-13, (xs[rel.argmax()], rel.max())
    assert np.median(rel) < 1e-14
    bad = np.array([0.0, -1.0])
    assert lib.vdr_diag_beta_vf(2, bad.ctypes.data_as(D), got.ctypes.data_as(D)) == 4
