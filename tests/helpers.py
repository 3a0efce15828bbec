"""Test helpers: the reference's recorded case built from the golden
fixture, and small problem factories."""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def load_kat():
    with open(os.path.join(GOLDEN, "vanadis_log_kat.json")) as f:
        return json.load(f)


def kat_problem(vdr, variant=None):
    """The 7x20x20 case of src_v2026_2_1/vanadis_log.txt."""
    k = load_kat()
    P = vdr.problems
    mesh = P.axis_mesh(k["dx"], k["dy"], k["dz"])
    c = k["cfg"]
    return P.uniform_fields_problem(
        "vanadis_log_7x20x20", mesh, lam=c["K"], pdec=c["P"],
        vel3=(c["V1"], c["V2"], c["V3"]), q_total=c["Q"],
        source_element=k["source_element_1based"], robin_alpha=c["ALPHA"],
        mask_mode=P.MASK_VF, variant=P.DR_VF if variant is None else variant,
        tol=k["tol"])


def run_kat_oracle(oracle, prob, steps=20, itmax=1000):
    """The reference's time loop (program vanadis + przest3d) on the oracle:
    returns per-step iterations, residuals and masses, and the dominance
    factor of the first step's element matrices."""
    k = load_kat()
    m = prob.mesh
    dt = float(k["dt"])
    t = np.zeros(m.nnode)
    its, errs, masses = [], [], []
    dom = None
    for step in range(steps):
        bb, b, diag = oracle.assemble(
            prob.variant, m.xx, m.yy, m.zz, m.iss, prob.vel, prob.lam,
            prob.pdec, prob.q, kod=m.kod, robin_alpha=prob.robin_alpha,
            aH=2.0, aM=3.0 / dt, cf=3.0, rM=3.0 / dt, t_old=t)
        if step == 0:
            dom = oracle.dominance_factor(m.iss, bb, m.nnode)
        bc = prob.bc
        b[bc == 1] = 0.0
        diag[bc == 1] = 1.0
        t[bc == 1] = 0.0
        t, it, err, st = oracle.dbcg(b, t, bb, m.iss, diag, bc, k["tol"], itmax)
        its.append(it)
        errs.append(err)
        masses.append(oracle.integrate_mass(m.iss, m.xx, m.yy, m.zz, t))
    return dict(iterations=its, residuals=errs, masses=masses, dominance=dom,
                solution=t)


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = float(np.max(np.abs(b))) if b.size else 0.0
    if not scale > 0.0 or not np.isfinite(scale):
        scale = 1.0
    nb = np.linalg.norm(b / scale)  # scaled: no overflow for |b| ~ 1e200
    return float(np.linalg.norm((a - b) / scale) / (nb if nb > 0 else 1.0))
