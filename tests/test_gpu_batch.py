"""Many independent meshes solved together (segmented BiCGStab) through the
C ABI: every mesh's solution against the single-mesh FP64 solve of the
same mesh, and its residual recomputed by the oracle; bad segment layouts
rejected on the host; meshes with zero right-hand side; the autotuned tile
shape."""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu


def theta(dt):
    return 2.0, 3.0 / dt


@pytest.fixture(scope="module")
def batch(vdr):
    P = vdr.problems
    probs = P.cube_batch(7, seed=2001, nmin=2, nmax=7)
    return probs, P.concat(probs)


def test_segmented_solve_matches_single_mesh_solves(vdr, oracle, gpu_lib, batch):
    import torch
    probs, union = batch
    aH, aM = theta(10.0 / 5)
    tol = 1e-11
    with vdr.Solver(union, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s:
        s.set_segments(union.mesh.node_off)
        b = torch.as_tensor(s.assemble_rhs(3.0, 0.0, None), device="cuda")
        x = torch.zeros_like(b)
        torch.cuda.synchronize()
        its, errs, sts, st = s.solve_segmented_device(b, x, tol=tol, itmax=5000)
        torch.cuda.synchronize()
        X, B = x.cpu().numpy(), b.cpu().numpy()
        tile, threads = s.segment_tuning()
    assert st == 0 and np.all(sts == 0) and np.all(errs <= tol), (its, errs, sts)
    assert tile in (512, 1024, 2048, 4096) and threads in (128, 256, 512)
    off = union.mesh.node_off
    for m, p in enumerate(probs):
        xm, bm = X[off[m]:off[m + 1]], B[off[m]:off[m + 1]]
        with vdr.Solver(p, vdr.Options(apply_mode="stored"), aH=aH, aM=aM) as s1:
            b1 = s1.assemble_rhs(3.0, 0.0, None)
            assert rel_l2(bm, b1) < 1e-13
            x1, it1, e1, st1 = s1.solve(b1, tol=tol, itmax=5000)
        assert st1 == 0
        assert rel_l2(xm, x1) < 1e-8, m
        assert abs(int(its[m]) - it1) <= 2, (m, its[m], it1)
        mm = p.mesh
        bb, _, _ = oracle.assemble(p.variant, mm.xx, mm.yy, mm.zz, mm.iss, p.vel,
                                   p.lam, p.pdec, p.q, kod=mm.kod, aH=aH, aM=aM,
                                   want_b=False, want_diag=False)
        ax, _ = oracle.matvec0(mm.iss, bb, p.bc, xm)
        assert rel_l2(ax, bm) <= 1.01 * tol, m


def test_segments_must_not_couple(vdr, gpu_lib, batch):
    probs, union = batch
    with vdr.Solver(union) as s:
        off = np.array(union.mesh.node_off).copy()
        off[2] += 1  # the boundary falls inside mesh 1
        with pytest.raises(vdr.VdrError) as ei:
            s.set_segments(off)
        assert ei.value.status == 4
        with pytest.raises(vdr.VdrError):
            s.set_segments([0, 5, 3, union.mesh.nnode])


def test_zero_rhs_segment(vdr, gpu_lib, batch):
    import torch
    probs, union = batch
    aH, aM = theta(2.0)
    with vdr.Solver(union, aH=aH, aM=aM) as s:
        s.set_segments(union.mesh.node_off)
        off = union.mesh.node_off
        bh = s.assemble_rhs(3.0, 0.0, None)
        bh[off[3]:off[4]] = 0.0
        b = torch.as_tensor(bh, device="cuda")
        x = torch.ones_like(b)
        torch.cuda.synchronize()
        its, errs, sts, st = s.solve_segmented_device(b, x, tol=1e-10)
        torch.cuda.synchronize()
        X = x.cpu().numpy()
    assert st == 0 and np.all(sts == 0)
    assert np.all(X[off[3]:off[4]] == 0.0) and errs[3] == 0.0 and its[3] == 0
