"""Oracle results for a synthetic problem (TEST INFRASTRUCTURE ONLY).

Given a problem object from the product's seeded generator (mesh arrays,
per-element fields, Dirichlet mask, DR variant), runs the CPU oracle to get
everything the GPU path is compared with: element matrices, right-hand
side, Jacobi diagonal, a seeded probe apply in both orientations and a
tightly converged solution.
"""
from __future__ import annotations

import numpy as np

from . import assemble, bicgstab, matvec0


def probe_vector(n: int, seed: int = 12345) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal(n)


def reference_system(prob, aH=1.0, aM=0.0, cf=1.0, rM=0.0, t_old=None,
                     solve=True, tol=1e-12, itmax=20000, seed=12345,
                     nthreads=1):
    m = prob.mesh
    bb, b, diag = assemble(prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                           prob.lam, prob.pdec, prob.q, kod=m.kod,
                           robin_alpha=prob.robin_alpha, aH=aH, aM=aM, cf=cf,
                           rM=rM, t_old=t_old, nthreads=nthreads)
    bc = prob.bc
    b[bc == 1] = 0.0
    diag[bc == 1] = 1.0
    xp = probe_vector(m.nnode, seed)
    yp, _ = matvec0(m.iss, bb, bc, xp)
    ytp, _ = matvec0(m.iss, bb, bc, xp, transpose=True)
    out = dict(bb=bb, b=b, diag=diag, x_probe=xp, y_probe=yp, yt_probe=ytp)
    if solve:
        x, it, err, st = bicgstab(b, np.zeros(m.nnode), bb, m.iss, diag, bc,
                                  tol=tol, itmax=itmax)
        out.update(x_solution=x, iterations=it, err=err, status=st)
    return out


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = float(np.max(np.abs(b))) if b.size else 0.0
    if not scale > 0.0 or not np.isfinite(scale):
        scale = 1.0
    nb = np.linalg.norm(b / scale)  # scaled: no overflow for |b| ~ 1e200
    return float(np.linalg.norm((a - b) / scale) / (nb if nb > 0 else 1.0))
