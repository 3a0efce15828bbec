"""The element build's geometric-factor form of el3d, restated in numpy and
checked against the oracle's el3d (the reference's operation order) on
jittered hexahedra, for the three DR variants (CPU):

    H_ij = lambda K_ij + sum_q detJ_q W_i(q) (a_j(q) + P N_j(q)),
    M_ij = sum_q detJ_q W_i(q) N_j(q),
    K_ij = sum_q detJ_q gradN_i . gradN_j       (geometry only),
    a_j(q) = (J_q^-1 v) . dN_j/dxi(q),  W_j(q) = N_j(q) + tau_q a_j(q),

A_e = aH H + aM M.  K, J^-1 and detJ are what the GPU keeps per mesh; the
rest is what every build forms from the fields.  Bar: 1e-13 relative (max
norm per element matrix); the two evaluations differ only in rounding.
"""
import numpy as np
import pytest

G = 0.577350269189626
SX = np.array([-1, 1, 1, -1, -1, 1, 1, -1], dtype=float)
SY = np.array([-1, -1, 1, 1, -1, -1, 1, 1], dtype=float)
SZ = np.array([-1, -1, -1, -1, 1, 1, 1, 1], dtype=float)
OT, GP, VF = 0, 1, 2


def shape(xi, eta, zeta):
    n = 0.125 * (1 + SX * xi) * (1 + SY * eta) * (1 + SZ * zeta)
    dn = np.stack([0.125 * SX * (1 + SY * eta) * (1 + SZ * zeta),
                   0.125 * SY * (1 + SX * xi) * (1 + SZ * zeta),
                   0.125 * SZ * (1 + SX * xi) * (1 + SY * eta)])
    return n, dn


def tau_at(variant, jinv, xe, ye, ze, lam, v):
    eps = 1e-14
    vmag = np.sqrt(v @ v)
    if variant == OT:
        dlx, dly, dlz = abs(xe[1] - xe[0]), abs(ye[3] - ye[0]), abs(ze[4] - ze[0])
        h = 2.0 / (abs(v[0]) / dlx + abs(v[1]) / dly + abs(v[2]) / dlz + eps) if vmag > eps else 0.0
        lams = lam
    else:
        e = v / vmag if vmag > eps else np.zeros(3)
        g = jinv @ e
        gn = np.sqrt(g @ g)
        h = 2.0 / gn if gn > eps else 0.0
        lams = lam * (e @ e) if variant == VF else lam
    pe = vmag * h / (2.0 * lams) if (vmag > eps and lams > eps) else 0.0
    if not (pe > 1e-12 and vmag > eps):
        return 0.0
    if variant == VF:
        if pe < 1e-3:
            beta = pe / 3 - pe ** 3 / 45 + 2 * pe ** 5 / 945
        elif pe > 50:
            beta = 1 - 1 / pe
        else:
            beta = 1 / np.tanh(pe) - 1 / pe
    else:
        beta = np.cosh(pe) / np.sinh(pe) - 1 / pe
    return 0.5 * h / vmag * beta


def element_geo_form(variant, xe, ye, ze, lam, pdec, v, aH, aM):
    X = np.stack([xe, ye, ze])
    K = np.zeros((8, 8))
    per_point = []
    for q in range(8):
        n, dn = shape(G * SX[q], G * SY[q], G * SZ[q])
        J = X @ dn.T                     # J[a][b] = d x_a / d xi_b
        detj = np.linalg.det(J)
        jinv = np.linalg.inv(J)          # jinv[a][b] = d xi_a / d x_b
        grad = jinv.T @ dn               # grad[d][j] = d N_j / d x_d
        K += detj * grad.T @ grad        # geometry only
        tau = tau_at(variant, jinv, xe, ye, ze, lam, v)
        a = (jinv @ v) @ dn              # v . grad N_j
        per_point.append((detj, n + tau * a, a, n))
    H = lam * K
    M = np.zeros((8, 8))
    for detj, w, a, n in per_point:
        H += detj * np.outer(w, a + pdec * n)
        M += detj * np.outer(w, n)
    return aH * H + aM * M


def random_hexes(E, seed):
    """E separate jittered unit-scale hexahedra (8 nodes each)."""
    rng = np.random.default_rng(seed)
    h = 10.0 ** rng.uniform(-3, 0, E)
    base = rng.uniform(-1, 1, (E, 3))
    xe = base[:, :1] + h[:, None] * (0.5 * (SX + 1) + 0.2 * rng.uniform(-1, 1, (E, 8)))
    ye = base[:, 1:2] + h[:, None] * (0.5 * (SY + 1) + 0.2 * rng.uniform(-1, 1, (E, 8)))
    ze = base[:, 2:] + h[:, None] * (0.5 * (SZ + 1) + 0.2 * rng.uniform(-1, 1, (E, 8)))
    v = rng.standard_normal((E, 3))
    # Peclet numbers ~0.05 .. 500 over the elements
    lam = np.sqrt((v ** 2).sum(1)) * h * 10.0 ** rng.uniform(-3, 1, E)
    return h, xe, ye, ze, v, lam


@pytest.mark.parametrize("variant", [OT, GP, VF])
def test_geometric_factor_form_equals_el3d(oracle, variant):
    E = 64
    _, xe, ye, ze, v, lam = random_hexes(E, 40 + variant)
    pdec = np.full(E, 0.3)
    aH, aM = 2.0, 7.0
    iss = (np.arange(8)[:, None] + 8 * np.arange(E)[None, :] + 1).astype(np.int32).ravel()
    xx, yy, zz = xe.ravel(), ye.ravel(), ze.ravel()
    vel = np.concatenate([v[:, 0], v[:, 1], v[:, 2]])
    bb, _, _ = oracle.assemble(variant, xx, yy, zz, iss, vel, lam, pdec, np.zeros(E),
                               kod=None, robin_alpha=0.0, aH=aH, aM=aM,
                               want_b=False, want_diag=False)
    bb = bb.reshape(E, 8, 8)
    worst = 0.0
    for e in range(E):
        A = element_geo_form(variant, xe[e], ye[e], ze[e], lam[e], pdec[e], v[e], aH, aM)
        worst = max(worst, np.abs(A - bb[e]).max() / np.abs(bb[e]).max())
    assert worst < 1e-13, worst
