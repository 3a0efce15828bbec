"""Parity at the benchmark's full size: the 256 x 256 x 128 rotation + shear
theta step (8,388,608 elements, 8,520,321 nodes; the bench's step), against
the oracle assembled and solved on all host cores.

* element matrices of the step's build (from the mesh's geometric factors)
  and of the build that evaluates the Jacobians from the coordinates,
  against the oracle's BB: 1e-12 relative L2, 1e-13 between the two;
* operator apply and its transpose: GPU vs the oracle's colour-parallel
  matvec_0 / mttvec_0 on the oracle's BB, 1e-12 relative L2, with the
  atomic scatter and with the colour-by-colour scatter;
* Jacobi diagonal and right-hand side: 1e-12;
* the solution of the step (both solved to 1e-12): 1e-9, with either
  scatter;
* size-independent identities on the GPU alone: linearity of the apply and
  the adjoint identity (A x, y) = (x, A^T y);
* the mixed-precision step (FP32 inner solves) at the FP64 tolerance, its
  true residual recomputed by the oracle;
* the 64-right-hand-side block solve at its full size (128 x 128 x 64):
  every column's true residual recomputed by the oracle;
* the 256-mesh segmented solve at its full size (8.17M elements): every
  mesh's true residual recomputed by the oracle.
"""
import os

import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

NEX, NEY, NEZ = 256, 256, 128
COURANT = 10.0


@pytest.fixture(scope="module")
def full(vdr, oracle):
    prob = vdr.problems.rotation_shear(NEX, NEY, NEZ, seed=1002)
    dt = COURANT / max(NEX, NEY, NEZ)
    aH, aM = 2.0, 3.0 / dt
    m = prob.mesh
    nt = os.cpu_count() or 1
    bb, b, d = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                               prob.lam, prob.pdec, prob.q, kod=m.kod,
                               robin_alpha=prob.robin_alpha, aH=aH, aM=aM,
                               cf=3.0, rM=aM, nthreads=nt)
    b[prob.bc == 1] = 0.0
    d[prob.bc == 1] = 1.0
    c, nc = oracle.greedy_colors(m.iss, m.nnode)
    colors = oracle.color_lists(c, nc)
    s = vdr.Solver(prob, vdr.Options(), aH=aH, aM=aM)
    yield {"prob": prob, "aH": aH, "aM": aM, "bb": bb, "b": b, "d": d,
           "colors": colors, "nt": nt, "s": s}
    s.close()


def test_fullsize_element_matrices_both_builds(gpu_lib, full):
    s = full["s"]
    bb_geo = s.element_matrices()
    assert s.geometry_status()[0] == 1
    assert rel_l2(bb_geo, full["bb"]) < 1e-12
    s.set_build_mode("recompute")
    try:
        bb_rc = s.element_matrices()
    finally:
        s.set_build_mode("auto")
    assert rel_l2(bb_rc, full["bb"]) < 1e-12
    assert rel_l2(bb_geo, bb_rc) < 1e-13


def test_fullsize_apply_parity(oracle, gpu_lib, full):
    prob, s = full["prob"], full["s"]
    m = prob.mesh
    x = np.random.default_rng(5).standard_normal(m.nnode)
    ce, co = full["colors"]
    for tr in (False, True):
        yref = oracle.matvec0_omp(m.iss, full["bb"], prob.bc, ce, co, x,
                                  transpose=tr, nthreads=full["nt"])
        assert rel_l2(s.apply(x, transpose=tr), yref) < 1e-12, tr


def test_fullsize_diag_and_rhs_parity(gpu_lib, full):
    s = full["s"]
    assert rel_l2(s.diag(), full["d"]) < 1e-12
    b = s.assemble_rhs(3.0, full["aM"], None)
    assert rel_l2(b, full["b"]) < 1e-12


def test_fullsize_solution_parity(oracle, gpu_lib, full):
    prob, s = full["prob"], full["s"]
    m = prob.mesh
    xr, itr, errr, st = oracle.bicgstab(full["b"], np.zeros(m.nnode), full["bb"],
                                        m.iss, full["d"], prob.bc, 1e-12, 20000,
                                        colors=full["colors"], nthreads=full["nt"])
    assert st == 0 and errr <= 1e-12
    x, it, err, st = s.solve(full["b"], tol=1e-12, itmax=20000)
    assert st == 0 and err <= 1e-12
    assert rel_l2(x, xr) < 1e-9
    assert abs(it - itr) <= max(3, 0.1 * itr), (it, itr)


@pytest.fixture(scope="module")
def full_color(vdr, full):
    """The same step on a handle with the colour-by-colour scatter (element
    storage in parity-colour order, one launch per colour, no atomics)."""
    s = vdr.Solver(full["prob"], vdr.Options(scatter="color"), aH=full["aH"],
                   aM=full["aM"])
    yield s
    s.close()


def test_fullsize_color_scatter_apply_parity(oracle, gpu_lib, full, full_color):
    prob = full["prob"]
    m = prob.mesh
    x = np.random.default_rng(6).standard_normal(m.nnode)
    ce, co = full["colors"]
    for tr in (False, True):
        yref = oracle.matvec0_omp(m.iss, full["bb"], prob.bc, ce, co, x,
                                  transpose=tr, nthreads=full["nt"])
        y = full_color.apply(x, transpose=tr)
        assert rel_l2(y, yref) < 1e-12, tr
        assert np.all(y[prob.bc == 1] == 0.0)


def test_fullsize_color_scatter_solution_parity(oracle, gpu_lib, full,
                                                full_color):
    """The colour-scatter step solved to the bench's tolerance (1e-8) and
    tightly (1e-12): its true residual recomputed by the oracle, and the
    tight solution against the oracle's BiCGStab at 1e-12."""
    prob = full["prob"]
    m = prob.mesh
    ce, co = full["colors"]
    assert rel_l2(full_color.diag(), full["d"]) < 1e-12
    assert rel_l2(full_color.assemble_rhs(3.0, full["aM"], None), full["b"]) < 1e-12
    x8, it8, err8, st8 = full_color.solve(full["b"], tol=1e-8, itmax=20000)
    assert st8 == 0 and err8 <= 1e-8
    r = full["b"] - oracle.matvec0_omp(m.iss, full["bb"], prob.bc, ce, co, x8,
                                       nthreads=full["nt"])
    assert np.linalg.norm(r) <= 1.01e-8 * np.linalg.norm(full["b"])
    xr, itr, errr, st = oracle.bicgstab(full["b"], np.zeros(m.nnode), full["bb"],
                                        m.iss, full["d"], prob.bc, 1e-12, 20000,
                                        colors=full["colors"], nthreads=full["nt"])
    assert st == 0 and errr <= 1e-12
    x, it, err, st = full_color.solve(full["b"], tol=1e-12, itmax=20000)
    assert st == 0 and err <= 1e-12
    assert rel_l2(x, xr) < 1e-9
    assert abs(it - itr) <= max(3, 0.1 * itr), (it, itr)


def test_fullsize_linearity_and_adjoint(gpu_lib, full):
    s = full["s"]
    n = full["prob"].mesh.nnode
    rng = np.random.default_rng(9)
    x, y = rng.standard_normal(n), rng.standard_normal(n)
    ax, ay = s.apply(x), s.apply(y)
    assert rel_l2(s.apply(2.0 * x - 3.0 * y), 2.0 * ax - 3.0 * ay) < 1e-13
    aty = s.apply(y, transpose=True)
    lhs, rhs = float(ax @ y), float(x @ aty)
    scale = np.linalg.norm(ax) * np.linalg.norm(y)
    assert abs(lhs - rhs) <= 1e-13 * scale, (lhs, rhs)


def test_fullsize_mixed_precision_step(oracle, gpu_lib, vdr, full):
    """Mixed precision at full size: FP64 refinement around FP32 inner solves
    reaches the FP64 true residual 1e-8 as the oracle measures it (its
    matvec_0 on its own BB), next to the FP64 solution."""
    prob = full["prob"]
    m = prob.mesh
    with vdr.Solver(prob, vdr.Options(precision="mixed"), aH=full["aH"],
                    aM=full["aM"]) as sm:
        x, it, err, st = sm.solve(full["b"], tol=1e-8, itmax=20000)
    assert st == 0 and err <= 1e-8
    ce, co = full["colors"]
    ax = oracle.matvec0_omp(m.iss, full["bb"], prob.bc, ce, co, x,
                            nthreads=full["nt"])
    r = full["b"] - ax
    assert np.linalg.norm(r) <= 1.01e-8 * np.linalg.norm(full["b"])
    x64, _, _, st64 = full["s"].solve(full["b"], tol=1e-8, itmax=20000)
    assert st64 == 0
    assert rel_l2(x, x64) < 1e-6


def test_fullsize_mixed_half_operator_step(oracle, gpu_lib, vdr, full):
    """The same step with the binary16 inner operator (P A P D^-1 per element,
    one power-of-two scale each): the FP64 true residual 1e-8 as the oracle
    measures it, next to the FP64 solution."""
    import torch
    prob = full["prob"]
    m = prob.mesh
    with vdr.Solver(prob, vdr.Options(), aH=full["aH"], aM=full["aM"]) as sm:
        sm.set_mixed_operator("half")
        b = torch.as_tensor(full["b"], device="cuda")
        x = torch.zeros_like(b)
        torch.cuda.synchronize()
        outer, inner, err, st = sm.solve_mixed_device(b, x, tol=1e-8,
                                                      inner_tol=1e-3)
        torch.cuda.synchronize()
        x = x.cpu().numpy()
    assert st == 0 and err <= 1e-8, (outer, inner, err)
    ce, co = full["colors"]
    ax = oracle.matvec0_omp(m.iss, full["bb"], prob.bc, ce, co, x,
                            nthreads=full["nt"])
    assert np.linalg.norm(full["b"] - ax) <= 1.01e-8 * np.linalg.norm(full["b"])
    x64, _, _, st64 = full["s"].solve(full["b"], tol=1e-8, itmax=20000)
    assert st64 == 0
    assert rel_l2(x, x64) < 1e-6


def test_fullsize_block_solve_residuals(oracle, gpu_lib, vdr):
    """Many right-hand sides at full size: 128 x 128 x 64 elements, K = 64 Gaussian
    sources, the refined block solve on the tensor-core block apply; every
    column's FP64 true residual, recomputed by the oracle, at 1e-8."""
    import torch
    prob = vdr.problems.rotation_shear(128, 128, 64, seed=1004)
    m = prob.mesh
    dt = COURANT / 128
    aH, aM = 2.0, 3.0 / dt
    nt = os.cpu_count() or 1
    bb, _, _ = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                               prob.lam, prob.pdec, prob.q, kod=m.kod,
                               robin_alpha=prob.robin_alpha, aH=aH, aM=aM,
                               want_b=False, want_diag=False, nthreads=nt)
    c, nc = oracle.greedy_colors(m.iss, m.nnode)
    ce, co = oracle.color_lists(c, nc)
    K = 64
    Q = vdr.problems.random_gaussian_sources(m, K)
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        Qd = torch.as_tensor(Q, device="cuda")
        Bd = torch.empty((m.nnode, K), dtype=torch.float64, device="cuda")
        s.assemble_rhs_block_device(Qd, Bd, 3.0)
        Xd = torch.zeros_like(Bd)
        no, ni, errs, st = s.solve_block_device(Bd, Xd, tol=1e-8, inner_tol=1e-4,
                                                precision="tf32x3")
        torch.cuda.synchronize()
        B, X = Bd.cpu().numpy(), Xd.cpu().numpy()
    assert st == 0 and np.all(errs <= 1e-8)
    for k in range(K):
        ax = oracle.matvec0_omp(m.iss, bb, prob.bc, ce, co, X[:, k], nthreads=nt)
        r = B[:, k] - ax
        assert np.linalg.norm(r) <= 1.01e-8 * np.linalg.norm(B[:, k]), k


def test_fullsize_segmented_meshes_residuals(oracle, gpu_lib, vdr):
    """Many meshes at full size: 256 cubes with edges of 8..48 elements
    (8.17M elements in all) in one segmented solve to 1e-8; every mesh's
    FP64 true residual, recomputed by the oracle on the union's BB, at
    1e-8."""
    import torch
    P = vdr.problems
    probs = P.cube_batch(256, seed=2001, nmin=8, nmax=48)
    union = P.concat(probs)
    m = union.mesh
    aH, aM = 2.0, 3.0 / (COURANT / 32.0)
    nt = os.cpu_count() or 1
    with vdr.Solver(union, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        s.set_segments(m.node_off)
        b = torch.as_tensor(s.assemble_rhs(3.0, 0.0, None), device="cuda")
        x = torch.zeros_like(b)
        torch.cuda.synchronize()
        its, errs, sts, st = s.solve_segmented_device(b, x, tol=1e-8, itmax=5000)
        torch.cuda.synchronize()
        X, B = x.cpu().numpy(), b.cpu().numpy()
    assert st == 0 and np.all(sts == 0) and np.all(errs <= 1e-8)
    bb, _, _ = oracle.assemble(union.variant, m.xx, m.yy, m.zz, m.iss, union.vel,
                               union.lam, union.pdec, union.q, kod=m.kod,
                               robin_alpha=union.robin_alpha, aH=aH, aM=aM,
                               want_b=False, want_diag=False, nthreads=nt)
    c, nc = oracle.greedy_colors(m.iss, m.nnode)
    ce, co = oracle.color_lists(c, nc)
    r = B - oracle.matvec0_omp(m.iss, bb, union.bc, ce, co, X, nthreads=nt)
    off = m.node_off
    for k in range(len(probs)):
        rk, bk = r[off[k]:off[k + 1]], B[off[k]:off[k + 1]]
        assert np.linalg.norm(rk) <= 1.01e-8 * np.linalg.norm(bk), k
