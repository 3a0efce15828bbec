"""The learned-preconditioner workload and its training pipeline.

Workload: the rotation + shear transport problem (lognormal diffusivity,
two Gaussian sources, zero Dirichlet on inflow faces) advanced by the
reference's theta scheme A = 2H + (3/dt)M, b = 3f - (H - (3/dt)M) T_old,
while the rotation axis tilts by a fixed angle per step (about the y axis),
so the velocity, the inflow mask and the operator change every step.  Each
step is solved to an FP64 relative residual of 1e-8.

Pipeline (every numerical step runs in libvdr on the GPU):
  1. the first `train_steps` steps are solved by Jacobi-BiCGStab with the
     iterates recorded (vdr_solve_record_device); each iterate x_k gives a
     pair (r, e) = (b - A x_k, x* - x_k) (vdr_net_make_pair_device);
  2. the network is trained on those pairs with Adam (the library's own
     forward and backward kernels, vdr_net_train_step_device), one pair per
     step, the features of the pair's time step loaded first;
  3. the remaining steps are solved twice from the same T_old -- plain
     Jacobi-BiCGStab and flexible BiCGStab right-preconditioned by the
     network (vdr_solve_learned_device, Jacobi on a stall) -- and the
     trajectory continues with the Jacobi solution.

Torch is used only to hold device buffers; its few buffer copies run on
the library's stream (the handle's stream does not synchronise with
torch's default stream).
"""
from __future__ import annotations

import math
import time

import numpy as np

from . import problems as P
from .solver import LearnedNet, Options, Solver


def tilted_velocity(mesh, step: int, tilt_deg: float = 0.5,
                    shear: float = 0.3, cents=None) -> np.ndarray:
    """Rotation about the axis (sin t, 0, cos t), t = tilt_deg * step,
    through the cube centre, plus the shear u_x += shear * z; scaled to
    max |u_e| = 1.  Step 0 is the rotation_shear field.  `cents`: the
    element centroids, if already computed."""
    cx, cy, cz = P.centroids(mesh) if cents is None else cents
    th = math.radians(tilt_deg * step)
    a = (math.sin(th), 0.0, math.cos(th))
    rx, ry, rz = cx - 0.5, cy - 0.5, cz - 0.5
    ux = a[1] * rz - a[2] * ry + shear * cz
    uy = a[2] * rx - a[0] * rz
    uz = a[0] * ry - a[1] * rx
    s = 1.0 / np.sqrt(ux * ux + uy * uy + uz * uz).max()
    return np.concatenate([ux * s, uy * s, uz * s])


class TiltingRun:
    """The transient problem on one Solver, T (the current field) on the
    device."""

    def __init__(self, nex, ney, nez, seed=1005, courant=10.0, tol=1e-8,
                 tilt_deg=0.5, device=0):
        import torch
        self.torch = torch
        self.prob = P.rotation_shear(nex, ney, nez, seed=seed)
        self.mesh = self.prob.mesh
        self.N = self.mesh.nnode
        self.dt = courant / max(nex, ney, nez)
        self.aH, self.aM = 2.0, 3.0 / self.dt
        self.cf, self.rM = 3.0, 3.0 / self.dt
        self.tol = tol
        self.tilt = tilt_deg
        self.cents = P.centroids(self.mesh)
        self.s = Solver(self.prob, Options(apply_mode="stored", device=device),
                        aH=self.aH, aM=self.aM)
        self.stream = torch.cuda.ExternalStream(self.s.stream())
        with torch.cuda.stream(self.stream):
            self.T = torch.zeros(self.N, dtype=torch.float64, device="cuda")
            self.b = torch.zeros_like(self.T)
        torch.cuda.synchronize()

    def set_step(self, step: int):
        """Fields, mask and operator of time step `step`; b from T."""
        p = self.prob
        vel = tilted_velocity(self.mesh, step, self.tilt, cents=self.cents)
        self.s.set_fields(vel, p.lam, p.pdec, p.q, p.robin_alpha)
        self.s.set_dirichlet(P.inflow_mask(self.mesh, vel))
        self.s.set_operator(self.aH, self.aM)
        self.s.assemble_rhs_device(self.b, self.cf, self.rM, self.T)

    def close(self):
        self.s.close()


def collect_pairs(run: TiltingRun, net: LearnedNet, steps, pairs_per_step,
                  max_iters=2000):
    """Solves `steps` (advancing run.T) recording iterates; returns the
    training set on the device: rhat [P][N], target [P][N] (float32),
    features [S][N][4], dbar [S], the index into `steps` of every pair, the
    Jacobi iteration counts and the steps."""
    torch = run.torch
    with torch.cuda.stream(run.stream):
        return _collect(run, net, steps, pairs_per_step, max_iters)


def _collect(run, net, steps, pairs_per_step, max_iters):
    torch = run.torch
    N = run.N
    S = len(steps)
    feats = torch.empty((S, N, 4), dtype=torch.float32, device="cuda")
    dbars = []
    rh, tg, owner, iters = [], [], [], []
    hist = torch.empty((max_iters + 1, N), dtype=torch.float64, device="cuda")
    for si, step in enumerate(steps):
        run.set_step(step)
        dbars.append(net.update_features(feats[si]))
        x = run.T.clone()
        x0 = run.T.clone()
        nh, it, err, st = run.s.solve_record_device(run.b, x, hist,
                                                    tol=run.tol,
                                                    itmax=max_iters)
        iters.append(it)
        # iterates: the start and x after each of the first it-1 iterations
        cands = [x0] + [hist[k] for k in range(min(nh, it) - 1)]
        take = np.unique(np.linspace(0, len(cands) - 1,
                                     min(pairs_per_step, len(cands)))
                         .round().astype(int))
        for k in take:
            r = torch.empty(N, dtype=torch.float32, device="cuda")
            t = torch.empty_like(r)
            net.make_pair(run.b, cands[k], x, r, t)
            rh.append(r)
            tg.append(t)
            owner.append(si)
        run.T.copy_(x)
    torch.cuda.synchronize()
    return dict(rhat=torch.stack(rh), target=torch.stack(tg), feats=feats,
                dbars=np.array(dbars), owner=np.array(owner), iters=iters,
                steps=list(steps))


def collect_pairs_learned(run: TiltingRun, net: LearnedNet, steps,
                          pairs_per_step, max_iters=60, restart=20):
    """The learned solver's own iterates: each step (T_old taken from the
    Jacobi-BiCGStab trajectory, which advances run.T) is solved by GCR with
    the current network, recording x_k; pairs (b - A x_k, x* - x_k) with x*
    the Jacobi-BiCGStab solution.  Same layout as collect_pairs."""
    torch = run.torch
    with torch.cuda.stream(run.stream):
        N = run.N
        S = len(steps)
        feats = torch.empty((S, N, 4), dtype=torch.float32, device="cuda")
        dbars, rh, tg, owner, iters = [], [], [], [], []
        hist = torch.empty((max_iters, N), dtype=torch.float64, device="cuda")
        for si, step in enumerate(steps):
            run.set_step(step)
            dbars.append(net.update_features(feats[si]))
            xs = run.T.clone()
            it, _, _ = run.s.solve_device(run.b, xs, tol=run.tol, itmax=5000)
            iters.append(it)
            x = run.T.clone()
            nh, itg, _, _ = run.s.solve_gcr_record_device(
                run.b, x, hist, net=net, tol=run.tol, itmax=max_iters,
                restart=restart)
            cands = [run.T] + [hist[k] for k in range(max(0, min(nh, itg) - 1))]
            take = np.unique(np.linspace(0, len(cands) - 1,
                                         min(pairs_per_step, len(cands)))
                             .round().astype(int))
            for k in take:
                r = torch.empty(N, dtype=torch.float32, device="cuda")
                t = torch.empty_like(r)
                net.make_pair(run.b, cands[k], xs, r, t)
                rh.append(r)
                tg.append(t)
                owner.append(si)
            run.T.copy_(xs)
        torch.cuda.synchronize()
        return dict(rhat=torch.stack(rh), target=torch.stack(tg), feats=feats,
                    dbars=np.array(dbars), owner=np.array(owner), iters=iters,
                    steps=list(steps))


def merge(a, b):
    """Union of two training sets collected on the same steps."""
    import torch
    assert a["steps"] == b["steps"]
    return dict(rhat=torch.cat([a["rhat"], b["rhat"]]),
                target=torch.cat([a["target"], b["target"]]),
                feats=a["feats"], dbars=a["dbars"],
                owner=np.concatenate([a["owner"], b["owner"]]),
                iters=a["iters"], steps=a["steps"])


def train(net: LearnedNet, data, epochs: int, lr: float = 1e-3,
          seed: int = 0, log_every: int = 0, loss: str = "residual",
          run: TiltingRun | None = None):
    """Adam over the pairs, one pair per optimizer step, cosine-decayed
    learning rate.  loss "residual": ||r - A M(r)|| / ||r|| with the
    operator of the pair's own time step (rebuilt on `run` when the step
    changes; pairs are visited step by step, steps and pairs in random
    order); loss "error": relative squared error against the target.
    Returns, per epoch, the mean loss of its last 10% of steps."""
    rh, tg, feats, dbars, owner = (data["rhat"], data["target"], data["feats"],
                                   data["dbars"], data["owner"])
    steps = data["steps"]
    rng = np.random.default_rng(seed)
    Pn = rh.shape[0]
    total = epochs * Pn
    k = 0
    curve = []
    by_step = [np.flatnonzero(owner == si) for si in range(len(steps))]
    for ep in range(epochs):
        losses = []
        if loss == "residual":
            order = []
            for si in rng.permutation(len(steps)):
                order.extend((si, pi) for pi in rng.permutation(by_step[si]))
        else:
            order = [(int(owner[pi]), pi) for pi in rng.permutation(Pn)]
        cur = -1
        for j, (si, pi) in enumerate(order):
            if si != cur:
                if loss == "residual":
                    run.set_step(steps[si])
                net.set_features(feats[si], float(dbars[si]))
                cur = si
            lr_k = lr * 0.5 * (1.0 + math.cos(math.pi * k / max(1, total)))
            want = j >= 0.9 * Pn
            if loss == "residual":
                l_k = net.train_step_residual(rh[pi], lr_k, want_loss=want)
            else:
                l_k = net.train_step(rh[pi], tg[pi], lr_k, want_loss=want)
            if want:
                losses.append(l_k)
            k += 1
        curve.append(float(np.mean(losses)) if losses else float("nan"))
        if log_every and (ep + 1) % log_every == 0:
            print("epoch %d loss %.4g" % (ep + 1, curve[-1]), flush=True)
    return curve


def evaluate(run: TiltingRun, net: LearnedNet, steps, itmax=5000,
             stall_window=20, method="gcr", restart=20):
    """Solves each step twice from the same T_old (Jacobi-BiCGStab, then
    the learned solve: restarted GCR, method "gcr"; flexible BiCGStab,
    "bicgstab"; or `restart` learned GCR steps then Jacobi-BiCGStab,
    "hybrid") and advances with the Jacobi solution."""
    torch = run.torch
    with torch.cuda.stream(run.stream):
        return _evaluate(run, net, steps, itmax, stall_window, method, restart)


def learned_solve(run, net, x, itmax, stall_window, method, restart):
    if method == "hybrid":
        return run.s.solve_learned_hybrid_device(net, run.b, x, tol=run.tol,
                                                 itmax=itmax,
                                                 learned_steps=restart)
    if method == "gcr":
        return run.s.solve_gcr_device(run.b, x, net=net, tol=run.tol,
                                      itmax=itmax, restart=restart,
                                      stall_window=stall_window)
    return run.s.solve_learned_device(net, run.b, x, tol=run.tol, itmax=itmax,
                                      stall_window=stall_window)


def _evaluate(run, net, steps, itmax, stall_window, method, restart):
    torch = run.torch
    out = []
    for step in steps:
        run.set_step(step)
        net.update_features()
        xj = run.T.clone()
        xl = run.T.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        itj, errj, stj = run.s.solve_device(run.b, xj, tol=run.tol, itmax=itmax)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        itl, errl, stl, fb = learned_solve(run, net, xl, itmax, stall_window,
                                           method, restart)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        true_l = run.s.true_residual_device(run.b, xl)
        diff = float(torch.linalg.norm(xl - xj) / torch.linalg.norm(xj))
        out.append(dict(step=step, jacobi_iters=itj, jacobi_s=t1 - t0,
                        jacobi_status=stj, learned_iters=itl,
                        learned_s=t2 - t1, learned_status=stl,
                        learned_true_residual=true_l, fell_back=fb,
                        rel_diff=diff))
        run.T.copy_(xj)
    return out
