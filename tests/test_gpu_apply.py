"""GPU operator parity against the oracle through the C ABI: the EBE DR
apply (stored element matrices and matrix-free recompute; atomic and colour
scatter; A and A^T), right-hand-side assembly, Jacobi diagonal and mass
integral.  Bar: 1e-12 relative L2 (FP64)."""
import numpy as np
import pytest

from helpers import kat_problem, rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12


def cases(vdr):
    P = vdr.problems
    out = {
        "const_adv_OT": P.constant_advection(8, 8, 4, seed=11),
        "rotation_VF": P.rotation_shear(9, 7, 5, seed=12),
        "rotation_GP": P.rotation_shear(7, 6, 5, seed=13, variant=P.DR_GP),
        "kat_VF_robin": kat_problem(vdr),
        "one_element": P.rotation_shear(1, 1, 1, seed=14),
        "ragged_2x1x3": P.rotation_shear(2, 1, 3, seed=15),
    }
    out["rotation_GP"].lam[:] = 0.02
    # decay and Robin on a jittered mesh
    p = P.rotation_shear(5, 4, 6, seed=16)
    p.pdec[:] = 0.3
    p.robin_alpha = 0.7
    out["rotation_decay_robin"] = p
    return out


@pytest.fixture(scope="module")
def problems(vdr):
    return cases(vdr)


CASE_NAMES = ["const_adv_OT", "rotation_VF", "rotation_GP", "kat_VF_robin",
              "one_element", "ragged_2x1x3", "rotation_decay_robin"]
MODES = [("stored", "atomic", "df"), ("stored", "color", "df"),
         ("stored", "warp", "df"),
         ("stored", "atomic", "fp64"), ("stored", "color", "fp64"),
         ("matrix_free", "atomic", "auto"), ("matrix_free", "color", "auto")]


def oracle_bb(oracle, prob, aH, aM):
    m = prob.mesh
    bb, _, _ = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                               prob.lam, prob.pdec, prob.q, kod=m.kod,
                               robin_alpha=prob.robin_alpha, aH=aH, aM=aM,
                               want_b=False, want_diag=False)
    return bb


@pytest.mark.parametrize("name", CASE_NAMES)
@pytest.mark.parametrize("mode,scatter,store", MODES)
def test_apply_parity(vdr, oracle, gpu_lib, problems, name, mode, scatter,
                      store):
    prob = problems[name]
    aH, aM = 2.0, 0.37
    bb = oracle_bb(oracle, prob, aH, aM)
    x = np.random.default_rng(5).standard_normal(prob.mesh.nnode)
    opts = vdr.Options(apply_mode=mode, scatter=scatter, matrix_storage=store)
    with vdr.Solver(prob, opts, aH=aH, aM=aM) as s:
        for tr in (False, True):
            yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc, x, transpose=tr)
            y = s.apply(x, transpose=tr)
            assert rel_l2(y, yref) < TOL, (name, mode, scatter, tr)
            assert np.all(y[prob.bc == 1] == 0.0)


@pytest.mark.parametrize("name", ["const_adv_OT", "kat_VF_robin",
                                  "rotation_decay_robin"])
def test_diag_and_rhs_parity(vdr, oracle, gpu_lib, problems, name):
    prob = problems[name]
    m = prob.mesh
    dt = 100.0
    aH, aM, cf, rM = 2.0, 3.0 / dt, 3.0, 3.0 / dt
    t_old = np.random.default_rng(6).standard_normal(m.nnode)
    t_old[prob.bc == 1] = 0.0
    _, b, d = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                              prob.lam, prob.pdec, prob.q, kod=m.kod,
                              robin_alpha=prob.robin_alpha, aH=aH, aM=aM,
                              cf=cf, rM=rM, t_old=t_old, want_bb=False)
    b[prob.bc == 1] = 0.0
    d[prob.bc == 1] = 1.0
    with vdr.Solver(prob, aH=aH, aM=aM) as s:
        assert rel_l2(s.diag(), d) < TOL
        assert rel_l2(s.assemble_rhs(cf, rM, t_old), b) < TOL
        # steady form: b = f
        _, bs, _ = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss,
                                   prob.vel, prob.lam, prob.pdec, prob.q,
                                   kod=m.kod, robin_alpha=prob.robin_alpha,
                                   want_bb=False, want_diag=False)
        bs[prob.bc == 1] = 0.0
        if np.linalg.norm(bs) > 0:
            assert rel_l2(s.assemble_rhs(1.0, 0.0, None), bs) < TOL


@pytest.mark.parametrize("scale", [1e-30, 1.0, 1e30])
def test_rhs_told_magnitudes(vdr, oracle, gpu_lib, problems, scale):
    """b = -(H - rM M) T_old (no source) for T_old of any magnitude, with
    zero nodes mixed in: the double-float build scales each element's T_old
    by a power of two, so it stays on its two launches (per-element DR
    scalars + build) without the FP64 redo."""
    import copy
    prob = copy.deepcopy(problems["rotation_decay_robin"])
    prob.q[:] = 0.0
    m = prob.mesh
    dt = 100.0
    aH, aM, cf, rM = 2.0, 3.0 / dt, 3.0, 3.0 / dt
    t_old = np.random.default_rng(8).standard_normal(m.nnode) * scale
    t_old[::3] = 0.0
    t_old[prob.bc == 1] = 0.0
    _, b, _ = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                              prob.lam, prob.pdec, prob.q, kod=m.kod,
                              robin_alpha=prob.robin_alpha, aH=aH, aM=aM,
                              cf=cf, rM=rM, t_old=t_old, want_bb=False,
                              want_diag=False)
    b[prob.bc == 1] = 0.0
    with vdr.Solver(prob, aH=aH, aM=aM) as s:
        s.diag()  # operator built
        n0 = vdr.kernel_launch_count()
        bg = s.assemble_rhs(cf, rM, t_old)
        launches = vdr.kernel_launch_count() - n0
    assert rel_l2(bg, b) < TOL
    assert launches == 2


def test_mass_parity(vdr, oracle, gpu_lib, problems):
    prob = problems["kat_VF_robin"]
    m = prob.mesh
    c = np.random.default_rng(7).random(m.nnode)
    ref = oracle.integrate_mass(m.iss, m.xx, m.yy, m.zz, c)
    with vdr.Solver(prob) as s:
        got = s.mass(c)
    assert abs(got - ref) <= 1e-12 * abs(ref)


def test_ot_variant_nan_semantics(vdr, oracle, gpu_lib):
    """OT's exp-based coth gives NaN above Pe = 709.78 in the reference; the
    GPU path reproduces it instead of silently differing."""
    prob = vdr.problems.constant_advection(4, 4, 2, seed=2)
    prob.lam[:] = 1e-7
    x = np.ones(prob.mesh.nnode)
    with vdr.Solver(prob, vdr.Options(apply_mode="stored")) as s:
        y = s.apply(x)
    assert np.isnan(y[prob.bc == 0]).any()


def test_bad_connectivity_rejected_on_host(vdr, gpu_lib):
    prob = vdr.problems.rotation_shear(2, 2, 2, seed=1)
    prob.mesh.iss = prob.mesh.iss.copy()
    prob.mesh.iss[3] = prob.mesh.nnode + 5
    with pytest.raises(vdr.VdrError) as ei:
        vdr.Solver(prob)
    assert ei.value.status == 4


@pytest.mark.parametrize("scale", [1e-300, 1e-200, 1e-40, 1.0, 1e40, 1e200])
def test_double_float_apply_any_input_scale(vdr, oracle, gpu_lib, problems,
                                            scale):
    """The double-float store scales each element's inputs by a power of two,
    so the apply keeps FP64 accuracy for vectors of any magnitude, including
    ones outside the FP32 range and mixed scales."""
    prob = problems["rotation_VF"]
    bb = oracle_bb(oracle, prob, 1.0, 0.0)
    rng = np.random.default_rng(6)
    x = rng.standard_normal(prob.mesh.nnode) * scale
    x[::7] *= 1e-30  # entries far below their neighbours
    with vdr.Solver(prob, vdr.Options(matrix_storage="df")) as s:
        for tr in (False, True):
            yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc, x, transpose=tr)
            assert rel_l2(s.apply(x, transpose=tr), yref) < TOL, (scale, tr)


def test_double_float_store_falls_back_outside_range(vdr, oracle, gpu_lib):
    """Operator entries beyond the pair store's exponent window (here
    diffusivity 1e45) send the operator to the FP64 store; results still
    match the oracle."""
    prob = vdr.problems.rotation_shear(4, 4, 3, seed=17)
    prob.lam[:] = 1e45
    bb = oracle_bb(oracle, prob, 1.0, 0.0)
    x = np.random.default_rng(7).standard_normal(prob.mesh.nnode)
    with vdr.Solver(prob, vdr.Options(matrix_storage="df")) as s:
        yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc, x)
        assert rel_l2(s.apply(x), yref) < TOL
