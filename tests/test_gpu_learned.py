"""The learned preconditioner on the GPU through the C ABI.

* forward pass and every parameter gradient of the network against the
  CPU float64 reference (oracle/unet_ref.py, autograd) with BF16 storage
  emulated: tolerances 1e-2 (output) and 3e-2 (gradients, relative L2 per
  layer) cover FP32 accumulation order and the BF16 rounding of activation
  gradients in the GPU's backward data pass;
* training on the GPU lowers the loss;
* an untrained network (zero head) is exactly Jacobi-BiCGStab;
* after training on the solver's own iterates (residual loss), on a later
  time step of the tilting-axis problem the network's preconditioner
  removes far more of a held-out residual than Jacobi, and every learned
  solve meets the FP64 tolerance.
"""
import numpy as np
import pytest

from helpers import rel_l2

pytestmark = pytest.mark.gpu


def dev(a):
    """Device copy, complete before returning (the library's stream does
    not wait for torch's)."""
    import torch
    t = torch.as_tensor(a, device="cuda")
    torch.cuda.synchronize()
    return t


def random_params(net_layout, n, seed):
    lay, total = net_layout
    assert total == n
    rng = np.random.default_rng(seed)
    p = np.zeros(n, dtype=np.float32)
    from oracle import unet_ref as U
    for i, (c1, c2, co, _) in enumerate(U.LAYERS):
        wo, bo, ws = lay[i]
        fan = 16 if i == U.HEAD else 27 * (c1 + c2)
        p[wo:wo + ws] = rng.standard_normal(ws) * np.sqrt(2.0 / fan)
        p[bo:bo + co] = 0.1 * rng.standard_normal(co)
    return p


@pytest.fixture(scope="module")
def small(vdr, gpu_lib):
    import torch
    prob = vdr.problems.rotation_shear(12, 10, 8, seed=51)
    s = vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=2.0, aM=30.0)
    net = vdr.LearnedNet(s, seed=3)
    feat = torch.empty((prob.mesh.nnode, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    dbar = net.update_features(feat)
    yield prob, s, net, feat, dbar
    net.close()
    s.close()


def test_param_layout_matches_reference(small):
    from oracle import unet_ref as U
    _, _, net, _, _ = small
    assert U.layout()[1] == net.nparam


def test_forward_matches_cpu(small):
    import torch
    from oracle import unet_ref as U
    prob, s, net, feat, dbar = small
    m = prob.mesh
    N = m.nnode
    p = random_params(U.layout(), net.nparam, 5)
    net.set_params(p)
    rh = np.random.default_rng(6).standard_normal(N).astype(np.float32)
    out = torch.empty(N, dtype=torch.float32, device="cuda")
    net.forward(dev(rh), out)
    torch.cuda.synchronize()
    theta = torch.tensor(p.astype(np.float64))
    ref = U.forward(theta, rh, feat.cpu().numpy(), m.nax, m.nay, m.naz)
    assert rel_l2(out.cpu().numpy(), ref.numpy()) < 1e-2


@pytest.fixture(scope="module")
def mid(vdr, gpu_lib):
    """A mesh whose coarsest level (11 x 19 x 3 nodes) still holds a whole
    TMA box of the tensor-core convolution (10 x 18 x 3 voxels)."""
    import torch
    prob = vdr.problems.rotation_shear(40, 72, 10, seed=53)
    s = vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=2.0, aM=30.0)
    net = vdr.LearnedNet(s, seed=4)
    feat = torch.empty((prob.mesh.nnode, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    net.update_features(feat)
    yield prob, s, net, feat
    net.close()
    s.close()


@pytest.mark.parametrize("mode", ["mma", "tcgen05"])
def test_forward_modes_match_cpu(mid, mode):
    """Both convolution paths -- tcgen05 (TMA halo slabs, TMEM accumulators)
    and warp-level mma.sync -- against the CPU float64 reference, 1e-2."""
    import torch
    from oracle import unet_ref as U
    prob, s, net, feat = mid
    m = prob.mesh
    N = m.nnode
    p = random_params(U.layout(), net.nparam, 11)
    net.set_params(p)
    net.set_conv(mode)
    rh = np.random.default_rng(12).standard_normal(N).astype(np.float32)
    out = torch.empty(N, dtype=torch.float32, device="cuda")
    net.forward(dev(rh), out)
    torch.cuda.synchronize()
    used, st = net.conv_status()
    assert (used, st) == (mode, 0)
    theta = torch.tensor(p.astype(np.float64))
    ref = U.forward(theta, rh, feat.cpu().numpy(), m.nax, m.nay, m.naz)
    assert rel_l2(out.cpu().numpy(), ref.numpy()) < 1e-2


def test_tcgen05_forward_matches_mma_at_c5_size(vdr, gpu_lib):
    """On the 128 x 128 x 64 mesh of the learned workload the tensor-core
    forward pass equals the mma.sync one up to BF16 rounding of the
    activations (both accumulate in FP32), and reports no timeout."""
    import torch
    from oracle import unet_ref as U
    prob = vdr.problems.rotation_shear(128, 128, 64, seed=1005)
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=2.0,
                    aM=30.0) as s:
        net = vdr.LearnedNet(s, seed=5)
        assert net.conv_status() == ("tcgen05", 0)   # the default
        net.update_features(None)
        net.set_params(random_params(U.layout(), net.nparam, 13))
        N = prob.mesh.nnode
        rh = dev(np.random.default_rng(14).standard_normal(N).astype(np.float32))
        outs = {}
        for mode in ("tcgen05", "mma", "tcgen05"):
            net.set_conv(mode)
            o = torch.empty(N, dtype=torch.float32, device="cuda")
            net.forward(rh, o)
            torch.cuda.synchronize()
            assert net.conv_status() == (mode, 0)
            if mode in outs:   # the same input twice: the same output
                assert torch.equal(outs[mode], o)
            outs[mode] = o
        a, b = outs["tcgen05"].cpu().numpy(), outs["mma"].cpu().numpy()
        assert np.all(np.isfinite(a))
        assert rel_l2(a, b) < 1e-2
        net.close()


def test_gradients_match_cpu(small):
    import torch
    from oracle import unet_ref as U
    prob, s, net, feat, dbar = small
    m = prob.mesh
    N = m.nnode
    p = random_params(U.layout(), net.nparam, 7)
    net.set_params(p)
    rng = np.random.default_rng(8)
    rh = rng.standard_normal(N).astype(np.float32)
    tg = rng.standard_normal(N).astype(np.float32)
    loss = net.loss_grad(dev(rh), dev(tg))
    g = net.get_grads()
    lref, gref, _ = U.loss_and_grad(p, rh, feat.cpu().numpy(), tg, prob.bc,
                                    m.nax, m.nay, m.naz)
    assert abs(loss - lref) <= 1e-2 * abs(lref)
    lay, _ = U.layout()
    for i, (wo, bo, ws) in enumerate(lay):
        co = U.LAYERS[i][2]
        for name, a, b in (("w", wo, wo + ws), ("b", bo, bo + co)):
            err = rel_l2(g[a:b], gref[a:b])
            assert err < 3e-2, (i, name, err)


def test_training_lowers_loss(small):
    import torch
    prob, s, net, feat, dbar = small
    N = prob.mesh.nnode
    from oracle import unet_ref as U
    net.set_params(random_params(U.layout(), net.nparam, 9))
    rng = np.random.default_rng(10)
    rh = dev(rng.standard_normal(N).astype(np.float32))
    tg = dev(np.sin(np.arange(N) / 17.0).astype(np.float32))
    first = net.loss_grad(rh, tg)
    for _ in range(60):
        net.train_step(rh, tg, 2e-3)
    last = net.loss_grad(rh, tg)
    assert last < 0.3 * first, (first, last)


def test_untrained_network_is_jacobi(vdr, gpu_lib):
    """The head starts at zero, so without post-smoothing the learned solve
    repeats the Jacobi solve's iterations."""
    import torch
    prob = vdr.problems.rotation_shear(10, 9, 7, seed=52)
    with vdr.Solver(prob, vdr.Options(apply_mode="stored"), aH=2.0,
                    aM=30.0) as s:
        net = vdr.LearnedNet(s, seed=1)
        net.set_smoothing(0)
        net.update_features()
        b = dev(s.assemble_rhs(1.0, 0.0, None))
        x1 = torch.zeros_like(b)
        x2 = torch.zeros_like(b)
        torch.cuda.synchronize()
        it1, e1, st1 = s.solve_device(b, x1, tol=1e-10)
        it2, e2, st2, fb = s.solve_learned_device(net, b, x2, tol=1e-10)
        assert st1 == 0 and st2 == 0 and not fb
        assert it1 == it2
        assert rel_l2(x2.cpu().numpy(), x1.cpu().numpy()) < 1e-12
        net.close()


def test_learned_preconditioner_gain(vdr, gpu_lib):
    """Train on the solver's own iterates of the first steps of the
    tilting-axis problem (residual loss), then on a later step: one
    application of the trained network's preconditioner removes far more of
    a held-out residual than Jacobi (the same preconditioner with an
    untrained network); the full learned solve (Jacobi-BiCGStab taking over
    on a stall) meets the FP64 tolerance and agrees with the plain solve.
    (Inside GCR the residuals soon leave the training distribution and the
    per-step gain fades; the benchmark reports whole solves as measured.)"""
    import torch
    L = vdr.learned
    run = L.TiltingRun(24, 24, 12, seed=1005, courant=10.0, tol=1e-8,
                       tilt_deg=3.0)
    net = vdr.LearnedNet(run.s, seed=11)
    jac = vdr.LearnedNet(run.s, seed=12)   # untrained: M = D^-1
    net.set_smoothing(0)
    jac.set_smoothing(0)
    data = L.collect_pairs(run, net, range(0, 6), pairs_per_step=30)
    curve = L.train(net, data, epochs=10, lr=1e-3, loss="residual", run=run)
    assert curve[-1] < 0.5
    held = L.collect_pairs(run, net, [6], pairs_per_step=10)
    run.set_step(6)
    net.update_features()
    jac.update_features()
    l_net = np.mean([net.residual_loss_grad(held["rhat"][i]) for i in range(10)])
    l_jac = np.mean([jac.residual_loss_grad(held["rhat"][i]) for i in range(10)])
    assert l_net < 0.3 * l_jac, (l_net, l_jac)
    out = L.evaluate(run, net, range(7, 9), method="gcr", stall_window=20)
    for r in out:
        assert r["jacobi_status"] == 0 and r["learned_status"] == 0, r
        assert r["learned_true_residual"] <= 1.05e-8, r
        assert r["rel_diff"] < 1e-5, r
    net.close()
    jac.close()
    run.close()
