"""The small plain-method configuration exactly as stated: a 32x32x16
jittered unit-cube HEX8 mesh (16,384 elements, 18,513 nodes, seed 1001),
constant velocity (1,0.5,0.25)/|.|, diffusivity 1e-3, a Gaussian source
(sigma 0.08) at (0.3,0.5,0.5), zero Dirichlet on inflow faces, the OT DR
variant (vanadis_full_DR_OpenMP_timing.for:1567-1716), the steady operator
A = H, FP64 Jacobi-preconditioned BiCGStab to 1e-10, greedy element
colouring.

Checked against the oracle at this size:
* the operator apply and its transpose in both scatter modes (atomic and
  colour-by-colour) and with warp-aggregated atomics, double-float and FP64
  stores and the matrix-free recompute: 1e-12 relative L2 (matvec_0 /
  mttvec_0, OT:1837-1933);
* the Jacobi diagonal and the right-hand side: 1e-12 (el3d + przest3d,
  OT:431-740);
* the greedy colouring: bit-exact against the oracle's first-fit greedy and
  the reference's parity formula (cudatest_coloring_gtx1060_optimized.cu:50-74);
* the solution of BiCGStab to 1e-10, every scatter mode: 1e-9 against the
  oracle's BiCG (dbcg_simple, OT:906-984) converged to 1e-13, and the
  iteration count against the oracle's BiCGStab at 1e-10;
* the reference's method (BiCG) on the GPU against the oracle's BiCG at 1e-10:
  iteration count and solution;
* the drop-in kernel_dbcg_simple_ on the oracle's BB at this size.
"""
import ctypes

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-10


@pytest.fixture(scope="module")
def c1(vdr, oracle):
    prob = vdr.problems.constant_advection()
    m = prob.mesh
    assert (m.nelem, m.nnode) == (16384, 18513)
    assert prob.variant == vdr.problems.DR_OT and prob.tol == TOL
    bb, b, d = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                               prob.lam, prob.pdec, prob.q, kod=m.kod,
                               robin_alpha=prob.robin_alpha, aH=1.0, aM=0.0,
                               cf=1.0, rM=0.0)
    b[prob.bc == 1] = 0.0
    d[prob.bc == 1] = 1.0
    x_tight, it_t, err_t, st_t = oracle.dbcg(b, np.zeros(m.nnode), bb, m.iss, d,
                                             prob.bc, 1e-13, 20000)
    assert st_t == 0
    return {"prob": prob, "bb": bb, "b": b, "d": d, "x": x_tight}


MODES = [("stored", "atomic", "df"), ("stored", "color", "df"),
         ("stored", "warp", "df"),
         ("stored", "atomic", "fp64"), ("stored", "color", "fp64"),
         ("matrix_free", "atomic", "auto"), ("matrix_free", "color", "auto")]


@pytest.mark.parametrize("mode,scatter,store", MODES)
def test_c1_apply_parity(vdr, oracle, gpu_lib, c1, mode, scatter, store):
    prob = c1["prob"]
    m = prob.mesh
    rng = np.random.default_rng(1001)
    opts = vdr.Options(apply_mode=mode, scatter=scatter, matrix_storage=store)
    with vdr.Solver(prob, opts) as s:
        for tr in (False, True):
            x = rng.standard_normal(m.nnode)
            yref, _ = oracle.matvec0(m.iss, c1["bb"], prob.bc, x, transpose=tr)
            y = s.apply(x, transpose=tr)
            assert rel_l2(y, yref) < 1e-12, (mode, scatter, store, tr)
            assert np.all(y[prob.bc == 1] == 0.0)


def test_c1_diag_and_rhs_parity(vdr, gpu_lib, c1):
    with vdr.Solver(c1["prob"]) as s:
        assert rel_l2(s.diag(), c1["d"]) < 1e-12
        assert rel_l2(s.assemble_rhs(1.0, 0.0, None), c1["b"]) < 1e-12


def test_c1_greedy_colouring_bit_exact(vdr, oracle, gpu_lib, c1):
    m = c1["prob"].mesh
    c_or, nc_or = oracle.greedy_colors(m.iss, m.nnode)
    colors = np.empty(m.nelem, dtype=np.int32)
    iss = np.ascontiguousarray(m.iss, dtype=np.int32)
    IP = ctypes.POINTER(ctypes.c_int)
    nc = gpu_lib.vdr_color_elements(m.nnode, m.nelem, iss.ctypes.data_as(IP),
                                    colors.ctypes.data_as(IP))
    assert nc == nc_or == 8
    assert np.array_equal(colors, np.asarray(c_or, dtype=np.int32))
    e = np.arange(m.nelem)
    i, j, k = e % 32, (e // 32) % 32, e // (32 * 32)
    assert np.array_equal(colors, (i & 1) + 2 * (j & 1) + 4 * (k & 1))


@pytest.mark.parametrize("scatter", ["atomic", "color", "warp"])
def test_c1_bicgstab_solution(vdr, oracle, gpu_lib, c1, scatter):
    prob = c1["prob"]
    m = prob.mesh
    _, it_ref, err_ref, st_ref = oracle.bicgstab(c1["b"], np.zeros(m.nnode),
                                                 c1["bb"], m.iss, c1["d"],
                                                 prob.bc, TOL, 20000)
    assert st_ref == 0 and err_ref <= TOL
    with vdr.Solver(prob, vdr.Options(solver="bicgstab", scatter=scatter)) as s:
        x, it, err, st = s.solve(c1["b"], tol=TOL, itmax=20000)
    assert st == 0 and err <= TOL
    ax, _ = oracle.matvec0(m.iss, c1["bb"], prob.bc, x)
    assert np.linalg.norm(c1["b"] - ax) <= 1.01 * TOL * np.linalg.norm(c1["b"])
    assert rel_l2(x, c1["x"]) < 1e-9
    assert abs(it - it_ref) <= max(3, 0.1 * it_ref), (it, it_ref)


@pytest.mark.parametrize("scatter", ["atomic", "color"])
def test_c1_bicg_matches_reference_method(vdr, oracle, gpu_lib, c1, scatter):
    prob = c1["prob"]
    m = prob.mesh
    x_ref, it_ref, err_ref, st_ref = oracle.dbcg(c1["b"], np.zeros(m.nnode),
                                                 c1["bb"], m.iss, c1["d"],
                                                 prob.bc, TOL, 20000)
    assert st_ref == 0
    with vdr.Solver(prob, vdr.Options(solver="bicg", scatter=scatter)) as s:
        x, it, err, st = s.solve(c1["b"], tol=TOL, itmax=20000)
    assert st == 0 and err <= TOL
    assert abs(it - it_ref) <= max(3, 0.05 * it_ref), (it, it_ref)
    assert rel_l2(x, x_ref) < 1e-8


def test_c1_dropin_kernel_dbcg_simple(vdr, oracle, gpu_lib, c1):
    prob = c1["prob"]
    m = prob.mesh
    x_ref, it_ref, _, st_ref = oracle.dbcg(c1["b"], np.zeros(m.nnode), c1["bb"],
                                           m.iss, c1["d"], prob.bc, TOL, 20000)
    assert st_ref == 0
    x, it, err = vdr.kernel_dbcg_simple(m.nnode, c1["b"], np.zeros(m.nnode), TOL,
                                        20000, c1["bb"], m.iss, c1["d"], m.nax,
                                        m.nay, m.naz, prob.bc)
    assert err <= TOL
    assert abs(it - it_ref) <= max(3, 0.05 * it_ref), (it, it_ref)
    assert rel_l2(x, x_ref) < 1e-8
    assert rel_l2(x, c1["x"]) < 1e-9
