"""GPU parity of the tcgen05 box block apply (VDR_BLOCK_APPLY_TCGEN05: 64
columns, 4 x 4 x 4-element box operators assembled in tensor memory and
multiplied with the boxes' node rows by tcgen05.mma kind::tf32).

The mesh is 42 x 37 x 21 elements: 11 x 10 x 6 = 660 boxes, about four per
CTA (so every stage and accumulator buffer of the kernel's pipeline turns
over), with partial boxes on the three upper faces.  Columns are compared
with the oracle's FP64 apply of the same FP32 inputs at the tolerances of
TF32 (2^-11 per operand) and split TF32, and with the mma.sync node tile.
"""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

TF32_TOL = {"tf32": 5e-3, "tf32x3": 2e-5}
K = 64


def to_dev(a, dtype):
    import torch
    t = torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")
    torch.cuda.synchronize()
    return t


@pytest.fixture(scope="module")
def big(vdr, oracle):
    prob = vdr.problems.rotation_shear(42, 37, 21, seed=71)
    aH, aM = 2.0, 3.0 * 42 / 10.0
    m = prob.mesh
    bb, _, _ = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                               prob.lam, prob.pdec, prob.q, kod=m.kod,
                               robin_alpha=prob.robin_alpha, aH=aH, aM=aM,
                               want_b=False, want_diag=False, nthreads=8)
    return prob, aH, aM, bb


def block_apply(vdr, prob, aH, aM, X, precision, variant, Y0=None):
    import torch
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        s.set_block_apply(variant)
        Xd = to_dev(X, torch.float32)
        if Y0 is None:
            Yd = torch.empty_like(Xd)
            s.apply_block_device(Xd, Yd, precision)
        else:
            Yd = to_dev(Y0, torch.float32)
            s.apply_block_accumulate_device(Xd, Yd, precision)
        torch.cuda.synchronize()
        return Yd.cpu().numpy().astype(np.float64)


@pytest.mark.parametrize("precision", ["tf32x3", "tf32"])
def test_tcgen05_apply_matches_oracle(vdr, oracle, gpu_lib, big, precision):
    prob, aH, aM, bb = big
    N = prob.mesh.nnode
    X = np.random.default_rng(72).standard_normal((N, K)).astype(np.float32)
    Y = block_apply(vdr, prob, aH, aM, X, precision, "tcgen05")
    worst = 0.0
    for k in (0, 1, 17, 32, 63):
        yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc, X[:, k].astype(np.float64))
        worst = max(worst, rel_l2(Y[:, k], yref))
    assert worst < TF32_TOL[precision], worst
    assert np.all(Y[prob.bc == 1] == 0.0)
    # the same product as the mma.sync node tile, to the split format's accuracy
    Yt = block_apply(vdr, prob, aH, aM, X, precision, "tile")
    assert rel_l2(Y.ravel(), Yt.ravel()) < 2 * TF32_TOL[precision]


def test_tcgen05_accumulate_ignores_dirichlet_entries(vdr, oracle, gpu_lib, big):
    """The accumulating call through the tcgen05 apply: Dirichlet rows of X
    read as zero whatever they hold (NaN, inf), Dirichlet rows of Y receive
    nothing, every other row gets A X added to what it held."""
    prob, aH, aM, bb = big
    N = prob.mesh.nnode
    d = prob.bc == 1
    rng = np.random.default_rng(73)
    X = rng.standard_normal((N, K)).astype(np.float32)
    X[d, 0::2] = np.nan
    X[d, 1::2] = np.inf
    # Y starts at the size of A X (a unit-size start would cost the FP32
    # sum more than the split format's accuracy in cancellation)
    Y0 = (1e-4 * rng.standard_normal((N, K))).astype(np.float32)
    Y0[d] = 7.0
    Y = block_apply(vdr, prob, aH, aM, X, "tf32x3", "tcgen05", Y0=Y0)
    assert np.all(Y[d] == 7.0)
    Xz = np.where(d[:, None], 0.0, X.astype(np.float64))
    for k in (0, 1, K - 1):
        yref, _ = oracle.matvec0(prob.mesh.iss, bb, prob.bc, Xz[:, k])
        got = np.where(d, 0.0, Y[:, k] - Y0[:, k].astype(np.float64))
        assert rel_l2(got, yref) < TF32_TOL["tf32x3"], k


def test_tcgen05_block_solve(vdr, oracle, gpu_lib, big):
    """A 64-column block solve with every inner apply on tcgen05: each
    column's FP64 residual, recomputed by the oracle, at the tolerance."""
    import torch
    prob, aH, aM, bb = big
    m = prob.mesh
    tol = 1e-8
    Q = vdr.problems.random_gaussian_sources(m, K, seed=74)
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        s.set_block_apply("tcgen05")
        Bd = torch.empty((m.nnode, K), dtype=torch.float64, device="cuda")
        s.assemble_rhs_block_device(to_dev(Q, torch.float64), Bd, 3.0)
        Xd = torch.zeros_like(Bd)
        no, ni, errs, st = s.solve_block_device(Bd, Xd, tol=tol, inner_tol=1e-4,
                                                precision="tf32x3")
        torch.cuda.synchronize()
        B, X = Bd.cpu().numpy(), Xd.cpu().numpy()
    assert st == 0 and np.all(errs <= tol), (st, errs)
    for k in (0, 21, K - 1):
        ax, _ = oracle.matvec0(m.iss, bb, prob.bc, X[:, k])
        assert rel_l2(ax, B[:, k]) <= 1.01 * tol, k
    assert np.all(X[prob.bc == 1] == 0.0)
