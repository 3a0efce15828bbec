"""Launch shapes chosen by measurement (vdr_apply_tuning): on a mesh large
enough to be tuned (64 x 64 x 32 = 131,072 elements) the stored apply, the
binary16 inner apply and the 64-column block apply (node-tile shapes and the
tcgen05 box apply) each pick one of their candidates with measured times,
and the operator keeps its parity with the oracle under the chosen shapes; a
small mesh keeps the defaults."""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu

GRIDS = [2, 4, 8, 16, 32]


def test_tuned_shapes_and_parity(vdr, oracle, gpu_lib):
    import torch
    prob = vdr.problems.rotation_shear(64, 64, 32, seed=61)
    m = prob.mesh
    aH, aM = 2.0, 30.0
    bb, _, d = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                               prob.lam, prob.pdec, prob.q, kod=m.kod,
                               robin_alpha=prob.robin_alpha, aH=aH, aM=aM,
                               want_b=False, nthreads=8)
    d[prob.bc == 1] = 1.0
    x = np.random.default_rng(62).standard_normal(m.nnode)
    with vdr.Solver(prob, vdr.Options(), aH=aH, aM=aM) as s:
        y = s.apply(x)                       # builds the operator, tunes
        t = s.apply_tuning()
        assert t["apply_blocks_per_sm"] in GRIDS
        assert all(v > 0 for v in t["apply_ms"].values())
        assert t["apply_ms"][t["apply_blocks_per_sm"]] <= min(t["apply_ms"].values()) + 1e-4
        yref, _ = oracle.matvec0(m.iss, bb, prob.bc, x)
        assert rel_l2(y, yref) < 1e-12
        # the binary16 inner operator, tuned when its store is first built
        s.set_mixed_operator("half")
        dx = torch.tensor(x, dtype=torch.float32, device="cuda")
        dy = torch.empty_like(dx)
        torch.cuda.synchronize()
        s.apply_half_device(dx, dy)
        torch.cuda.synchronize()
        t = s.apply_tuning()
        assert t["half_blocks_per_sm"] in GRIDS
        assert all(v > 0 for v in t["half_ms"].values())
        yh, _ = oracle.matvec0(m.iss, bb, prob.bc, x / d)
        assert rel_l2(dy.cpu().numpy().astype(np.float64), yh) < 2e-3
        # the block apply, tuned by the first 64-column block solve
        K = 64
        Q = vdr.problems.random_gaussian_sources(m, K)
        Qd = torch.as_tensor(Q, device="cuda")
        B = torch.empty((m.nnode, K), dtype=torch.float64, device="cuda")
        s.assemble_rhs_block_device(Qd, B, 3.0)
        X = torch.zeros_like(B)
        no, ni, errs, st = s.solve_block_device(B, X, tol=1e-8, inner_tol=1e-4,
                                                precision="tf32x3")
        torch.cuda.synchronize()
        assert st == 0 and np.all(errs <= 1e-8)
        t = s.apply_tuning()
        assert (t["block_tile_y"], t["block_halves"]) in [(2, 2), (2, 1), (4, 2)]
        assert all(v > 0 for v in t["block_ms"].values())
        assert set(t["block_ms"]) == {"2x2", "2x1", "4x2", "tcgen05"}
        # the tcgen05 box apply is chosen exactly when it timed fastest
        fastest = min(t["block_ms"], key=t["block_ms"].get)
        assert t["block_tcgen05"] == (fastest == "tcgen05")


def test_small_mesh_keeps_defaults(vdr, gpu_lib):
    prob = vdr.problems.rotation_shear(16, 16, 8, seed=63)
    with vdr.Solver(prob) as s:
        s.apply(np.ones(prob.mesh.nnode))
        t = s.apply_tuning()
    assert t["apply_blocks_per_sm"] == 8 and t["half_blocks_per_sm"] == 8
    assert (t["block_tile_y"], t["block_halves"]) == (2, 2) and not t["block_tcgen05"]
    assert all(v == 0 for v in t["apply_ms"].values())
