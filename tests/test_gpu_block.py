"""GPU parity of the many-right-hand-side path through the C ABI.

* block apply, FP64-accurate (double-float and FP64 stores): every column
  against the oracle's apply of that column, 1e-12 relative L2;
* block apply on the tensor cores (TF32, split TF32) against the oracle's
  FP64 apply of the same FP32 inputs, with the tolerances of those formats;
* block right-hand side: each column against the oracle's assembly of that
  column's source, 1e-12;
* the refined block solve: every column's FP64 residual, recomputed by the
  oracle, at the requested tolerance, and the solution against the
  single-right-hand-side FP64 solve.
"""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

COURANT = 10.0


def theta_case(vdr, nx, ny, nz, seed):
    """Rotation + shear field on a small mesh with the theta-step operator
    A = 2H + (3/dt)M at Courant number 10."""
    prob = vdr.problems.rotation_shear(nx, ny, nz, seed=seed)
    dt = COURANT / max(nx, ny, nz)
    return prob, 2.0, 3.0 / dt


def oracle_bb(oracle, prob, aH, aM):
    m = prob.mesh
    bb, _, _ = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                               prob.lam, prob.pdec, prob.q, kod=m.kod,
                               robin_alpha=prob.robin_alpha, aH=aH, aM=aM,
                               want_b=False, want_diag=False)
    return bb


def to_dev(a, dtype):
    """Device copy, complete before returning (the library's stream does
    not wait for torch's)."""
    import torch
    t = torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")
    torch.cuda.synchronize()
    return t


@pytest.fixture(scope="module")
def case(vdr, oracle):
    prob, aH, aM = theta_case(vdr, 9, 7, 6, seed=31)
    return prob, aH, aM, oracle_bb(oracle, prob, aH, aM)


@pytest.mark.parametrize("K", [1, 5, 16, 64])
@pytest.mark.parametrize("store,scatter", [("df", "atomic"), ("df", "color"),
                                           ("fp64", "atomic")])
def test_block_apply_fp64_parity(vdr, oracle, gpu_lib, case, K, store, scatter):
    import torch
    prob, aH, aM, bb = case
    N = prob.mesh.nnode
    X = np.random.default_rng(K).standard_normal((N, K))
    opts = vdr.Options(apply_mode="stored", scatter=scatter,
                       matrix_storage=store)
    with vdr.Solver(prob, opts, aH=aH, aM=aM) as s:
        Xd = to_dev(X, torch.float64)
        Yd = torch.empty_like(Xd)
        s.apply_block_device(Xd, Yd, "fp64")
        torch.cuda.synchronize()
        Y = Yd.cpu().numpy()
    for k in range(K):
        yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc, X[:, k])
        assert rel_l2(Y[:, k], yref) < 1e-12, k
    assert np.all(Y[prob.bc == 1] == 0.0)


# TF32 keeps 10 mantissa bits (relative rounding 2^-11 per operand); the
# split form drops only the tail-by-tail product (2^-22) and rounds in
# FP32 accumulation.
TF32_TOL = {"tf32": 5e-3, "tf32x3": 2e-5}


@pytest.mark.parametrize("K", [16, 32, 64])
@pytest.mark.parametrize("precision", ["tf32", "tf32x3"])
@pytest.mark.parametrize("variant", ["bulk", "lsu", "tile", "tcgen05"])
def test_block_apply_tensor_core(vdr, oracle, gpu_lib, case, K, precision,
                                 variant):
    import torch
    prob, aH, aM, bb = case
    N = prob.mesh.nnode
    X = np.random.default_rng(100 + K).standard_normal((N, K)).astype(np.float32)
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        s.set_block_apply(variant)
        Xd = to_dev(X, torch.float32)
        Yd = torch.empty_like(Xd)
        s.apply_block_device(Xd, Yd, precision)
        torch.cuda.synchronize()
        Y = Yd.cpu().numpy().astype(np.float64)
    worst = 0.0
    for k in range(K):
        yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc,
                                 X[:, k].astype(np.float64))
        worst = max(worst, rel_l2(Y[:, k], yref))
    assert worst < TF32_TOL[precision], worst
    assert np.all(Y[prob.bc == 1] == 0.0)


@pytest.mark.parametrize("precision,K", [("fp64", 5), ("tf32x3", 64)])
def test_block_apply_accumulate(vdr, oracle, gpu_lib, case, precision, K):
    """vdr_apply_block_accumulate_device adds P A P X into Y without zeroing
    it: two calls on a zero Y give twice the oracle's apply."""
    import torch
    prob, aH, aM, bb = case
    N = prob.mesh.nnode
    dt = torch.float64 if precision == "fp64" else torch.float32
    X = np.random.default_rng(55).standard_normal((N, K))
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        Xd = to_dev(X, dt)
        Yd = torch.zeros_like(Xd)
        s.apply_block_accumulate_device(Xd, Yd, precision)
        s.apply_block_accumulate_device(Xd, Yd, precision)
        torch.cuda.synchronize()
        Y = Yd.cpu().numpy().astype(np.float64)
    tol = 1e-12 if precision == "fp64" else TF32_TOL[precision]
    Xr = Xd.cpu().numpy().astype(np.float64)
    for k in (0, K - 1):
        yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc, Xr[:, k])
        assert rel_l2(Y[:, k], 2.0 * yref) < tol, k


@pytest.mark.parametrize("variant", ["tile", "lsu", "tcgen05"])
def test_block_apply_ignores_dirichlet_entries(vdr, oracle, gpu_lib, case,
                                               variant):
    """Dirichlet rows of X read as zero whatever they hold (NaN, inf) and
    Dirichlet rows of Y receive nothing (the accumulating call leaves them
    as they were)."""
    import torch
    prob, aH, aM, bb = case
    N, K = prob.mesh.nnode, 64
    d = prob.bc == 1
    X = np.random.default_rng(31).standard_normal((N, K)).astype(np.float32)
    X[d, 0::2] = np.nan
    X[d, 1::2] = np.inf
    Y0 = np.zeros((N, K), dtype=np.float32)
    Y0[d] = 7.0
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        s.set_block_apply(variant)
        Xd = to_dev(X, torch.float32)
        Yd = to_dev(Y0, torch.float32)
        s.apply_block_accumulate_device(Xd, Yd, "tf32x3")
        torch.cuda.synchronize()
        Y = Yd.cpu().numpy().astype(np.float64)
    assert np.all(Y[d] == 7.0)
    Xz = np.where(d[:, None], 0.0, X.astype(np.float64))
    for k in (0, 1, K - 1):
        yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc, Xz[:, k])
        assert rel_l2(np.where(d, 0.0, Y[:, k]), yref) < TF32_TOL["tf32x3"], k


def shuffled_elements(vdr, prob, seed):
    """The same problem with its elements in a random order (the node
    numbering is kept), so the mesh is no longer in the canonical structured
    numbering."""
    import dataclasses
    m = prob.mesh
    E = m.nelem
    perm = np.random.default_rng(seed).permutation(E)
    mesh = dataclasses.replace(
        m, iss=np.ascontiguousarray(m.iss.reshape(8, E)[:, perm]).ravel(),
        kod=np.ascontiguousarray(m.kod.reshape(6, E)[:, perm]).ravel())
    return dataclasses.replace(
        prob, mesh=mesh,
        vel=np.ascontiguousarray(prob.vel.reshape(3, E)[:, perm]).ravel(),
        lam=prob.lam[perm], pdec=prob.pdec[perm], q=prob.q[perm])


@pytest.mark.parametrize("layout", ["shuffled", "color"])
def test_block_apply_tile_request_off_the_structured_order(vdr, oracle, gpu_lib,
                                                           case, layout):
    """The node-tile variant needs the canonical structured numbering in
    storage order; on a shuffled element order or the colour-ordered store
    the request falls back to the per-element apply, with the same result."""
    import torch
    prob, aH, aM, bb = case
    opts = vdr.Options(apply_mode="stored")
    if layout == "shuffled":
        prob = shuffled_elements(vdr, prob, seed=5)
        bb = oracle_bb(oracle, prob, aH, aM)
    else:
        opts = vdr.Options(apply_mode="stored", scatter="color")
    N = prob.mesh.nnode
    X = np.random.default_rng(77).standard_normal((N, 32)).astype(np.float32)
    with vdr.Solver(prob, opts, aH=aH, aM=aM) as s:
        s.set_block_apply("tile")
        Xd = to_dev(X, torch.float32)
        Yd = torch.empty_like(Xd)
        s.apply_block_device(Xd, Yd, "tf32x3")
        torch.cuda.synchronize()
        Y = Yd.cpu().numpy().astype(np.float64)
    for k in (0, 31):
        yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc,
                                 X[:, k].astype(np.float64))
        assert rel_l2(Y[:, k], yref) < TF32_TOL["tf32x3"], k
    assert np.all(Y[prob.bc == 1] == 0.0)


def test_bounded_wait_times_out_and_recovers(vdr, oracle, gpu_lib, case):
    """The bulk-copy block apply's device waits are bounded: a wait that
    nothing completes gives up after its budget, the flag reaches the host
    as VDR_TIMEOUT, and the handle keeps working (a bulk-copy block apply
    afterwards matches the oracle)."""
    import importlib
    import torch
    L = importlib.import_module(vdr.__name__ + "._lib")
    prob, aH, aM, bb = case
    N = prob.mesh.nnode
    X = np.random.default_rng(9).standard_normal((N, 16)).astype(np.float32)
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        assert s.lib.vdr_diag_wait_timeout(s.h) == L.TIMEOUT
        s.set_block_apply("bulk")
        Xd = to_dev(X, torch.float32)
        Yd = torch.empty_like(Xd)
        s.apply_block_device(Xd, Yd, "tf32x3")
        torch.cuda.synchronize()
        Y = Yd.cpu().numpy().astype(np.float64)
    yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc, X[:, 0].astype(np.float64))
    assert rel_l2(Y[:, 0], yref) < TF32_TOL["tf32x3"]


def test_split_tf32_beats_tf32(vdr, oracle, gpu_lib, case):
    import torch
    prob, aH, aM, bb = case
    N = prob.mesh.nnode
    X = np.random.default_rng(7).standard_normal((N, 16)).astype(np.float32)
    yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc,
                             X[:, 3].astype(np.float64))
    errs = {}
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        for prec in ("tf32", "tf32x3"):
            Xd = to_dev(X, torch.float32)
            Yd = torch.empty_like(Xd)
            s.apply_block_device(Xd, Yd, prec)
            torch.cuda.synchronize()
            errs[prec] = rel_l2(Yd.cpu().numpy()[:, 3].astype(np.float64), yref)
    assert errs["tf32x3"] < errs["tf32"] / 30.0, errs


@pytest.mark.parametrize("scatter", ["atomic", "color"])
def test_block_rhs_parity(vdr, oracle, gpu_lib, case, scatter):
    import torch
    prob, aH, aM, _ = case
    m = prob.mesh
    K = 5
    Q = vdr.problems.random_gaussian_sources(m, K, seed=41)
    Q[2] *= 1e-150  # a tiny source
    Q[4] = 0.0      # and none
    cf = 3.0
    with vdr.Solver(prob, vdr.Options(scatter=scatter), aH=aH, aM=aM) as s:
        Bd = torch.empty((m.nnode, K), dtype=torch.float64, device="cuda")
        s.assemble_rhs_block_device(to_dev(Q, torch.float64), Bd, cf)
        torch.cuda.synchronize()
        B = Bd.cpu().numpy()
    for k in range(K):
        _, b, _ = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss,
                                  prob.vel, prob.lam, prob.pdec, Q[k],
                                  kod=m.kod, robin_alpha=prob.robin_alpha,
                                  aH=aH, aM=aM, cf=cf, want_bb=False,
                                  want_diag=False)
        b[prob.bc == 1] = 0.0
        if k == 4:
            assert np.all(B[:, k] == 0.0)
        else:
            assert rel_l2(B[:, k], b) < 1e-12, k


def column_residuals(oracle, prob, bb, B, X):
    """Per-column ||B - A X|| / ||B|| with the oracle's apply (norms of
    max-scaled vectors: columns near 1e200 do not overflow)."""
    out = []
    for k in range(B.shape[1]):
        ax, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc, X[:, k])
        r = B[:, k] - ax
        bm = np.max(np.abs(B[:, k]))
        rm = np.max(np.abs(r))
        if bm == 0.0:
            out.append(rm)
        elif rm == 0.0:
            out.append(0.0)
        else:
            out.append(rm * np.linalg.norm(r / rm) /
                       (bm * np.linalg.norm(B[:, k] / bm)))
    return np.array(out)


@pytest.mark.parametrize("precision,variant", [("tf32x3", "bulk"),
                                               ("tf32", "bulk"),
                                               ("tf32x3", "lsu"),
                                               ("tf32x3", "tile"),
                                               ("tf32", "tile")])
def test_block_solve_parity(vdr, oracle, gpu_lib, case, precision, variant):
    import torch
    prob, aH, aM, bb = case
    m = prob.mesh
    K, tol = 16, 1e-10
    Q = vdr.problems.random_gaussian_sources(m, K, seed=43)
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        s.set_block_apply(variant)
        Bd = torch.empty((m.nnode, K), dtype=torch.float64, device="cuda")
        s.assemble_rhs_block_device(to_dev(Q, torch.float64), Bd, 3.0)
        Xd = torch.zeros_like(Bd)
        no, ni, errs, st = s.solve_block_device(Bd, Xd, tol=tol,
                                                precision=precision)
        torch.cuda.synchronize()
        B, X = Bd.cpu().numpy(), Xd.cpu().numpy()
        # single right-hand-side FP64 solves of two columns
        singles = {k: s.solve(B[:, k], tol=1e-12, itmax=5000)[0]
                   for k in (0, K - 1)}
    assert st == 0 and no >= 1 and ni >= 1
    assert np.all(errs <= tol), errs
    res = column_residuals(oracle, prob, bb, B, X)
    assert np.all(res <= 1.01 * tol), res
    assert np.all(X[prob.bc == 1] == 0.0)
    for k, xs in singles.items():
        assert rel_l2(X[:, k], xs) < 1e-8, k


def test_block_solve_scaled_and_zero_columns(vdr, oracle, gpu_lib, case):
    """Columns of any magnitude converge (the FP32 inner right-hand side is
    a power-of-two-scaled copy of each column's residual); a zero column
    stays zero; a nonzero initial guess is refined."""
    import torch
    prob, aH, aM, bb = case
    N = prob.mesh.nnode
    K, tol = 16, 1e-10
    rng = np.random.default_rng(9)
    B = rng.standard_normal((N, K))
    B[prob.bc == 1] = 0.0
    B[:, 1] *= 1e-200
    B[:, 2] *= 1e200
    B[:, 3] *= 1e-30
    B[:, 5] = 0.0
    X0 = np.zeros((N, K))
    X0[:, 6] = rng.standard_normal(N)
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        Bd = to_dev(B, torch.float64)
        Xd = to_dev(X0, torch.float64)
        no, ni, errs, st = s.solve_block_device(Bd, Xd, tol=tol)
        torch.cuda.synchronize()
        X = Xd.cpu().numpy()
    assert st == 0, (st, errs)
    assert np.all(X[:, 5] == 0.0) and errs[5] == 0.0
    res = column_residuals(oracle, prob, bb, B, X)
    assert np.all(res <= 1.01 * tol), res


def test_block_bad_arguments(vdr, gpu_lib, case):
    import torch
    prob, aH, aM, _ = case
    N = prob.mesh.nnode
    with vdr.Solver(prob, aH=aH, aM=aM) as s:
        B = torch.zeros((N, 17), dtype=torch.float64, device="cuda")
        with pytest.raises(vdr.VdrError) as ei:
            s.solve_block_device(B, torch.zeros_like(B))
        assert ei.value.status == 4
        X = torch.zeros((N, 17), dtype=torch.float32, device="cuda")
        with pytest.raises(vdr.VdrError):
            s.apply_block_device(X, torch.zeros_like(X), "tf32")
