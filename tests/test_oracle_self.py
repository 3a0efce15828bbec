"""Self-consistency of the oracle beyond the recorded run: dense-matrix
cross-check of the EBE applies, transpose identity, agreement of the DR
variants where their streamline lengths coincide, the OT variant's
overflow, and agreement of the two Krylov methods."""
import numpy as np
import pytest

from helpers import rel_l2


def small_problem(vdr, variant=2, nex=4, ney=3, nez=3, jitter=0.1):
    P = vdr.problems
    prob = P.rotation_shear(nex, ney, nez, seed=77, variant=variant)
    return prob


def dense_from_bb(iss, bb, n):
    E = len(bb) // 64
    A = np.zeros((n, n))
    nd = iss.reshape(8, E) - 1
    for e in range(E):
        blk = bb[64 * e:64 * e + 64].reshape(8, 8)
        A[np.ix_(nd[:, e], nd[:, e])] += blk
    return A


@pytest.mark.parametrize("variant", [0, 1, 2])
def test_ebe_apply_equals_dense(vdr, oracle, variant):
    prob = small_problem(vdr)
    prob.lam[:] = 0.05  # keep OT finite
    m = prob.mesh
    bb, _, _ = oracle.assemble(variant, m.xx, m.yy, m.zz, m.iss, prob.vel,
                               prob.lam, prob.pdec, prob.q, kod=m.kod,
                               robin_alpha=0.3, aH=2.0, aM=0.7)
    A = dense_from_bb(m.iss, bb, m.nnode)
    P = np.diag(1.0 - prob.bc)
    x = np.random.default_rng(1).standard_normal(m.nnode)
    y, xm = oracle.matvec0(m.iss, bb, prob.bc, x)
    assert rel_l2(y, P @ A @ P @ x) < 1e-13
    assert np.all(xm[prob.bc == 1] == 0)
    yt, _ = oracle.matvec0(m.iss, bb, prob.bc, x, transpose=True)
    assert rel_l2(yt, P @ A.T @ P @ x) < 1e-13


def test_transpose_identity(vdr, oracle):
    prob = small_problem(vdr, nex=6, ney=5, nez=4)
    m = prob.mesh
    bb, _, _ = oracle.assemble(2, m.xx, m.yy, m.zz, m.iss, prob.vel, prob.lam,
                               prob.pdec, prob.q, kod=m.kod)
    rng = np.random.default_rng(2)
    x, y = rng.standard_normal(m.nnode), rng.standard_normal(m.nnode)
    ax, _ = oracle.matvec0(m.iss, bb, prob.bc, x)
    aty, _ = oracle.matvec0(m.iss, bb, prob.bc, y, transpose=True)
    assert abs(ax @ y - x @ aty) <= 1e-12 * abs(ax @ y)


def test_variants_coincide_on_bricks(oracle):
    """Undistorted brick, axis-aligned v with |v| = 2: OT's axis streamline
    length 2/(|v_y|/dly) equals the inverse-Jacobian length dly, so OT, GP
    and VF give the same element matrices."""
    xn = np.array([0, 2, 2, 0, 0, 2, 2, 0], float) * 0.5
    yn = np.array([0, 0, 1, 1, 0, 0, 1, 1], float) * 3.0
    zn = np.array([0, 0, 0, 0, 1, 1, 1, 1], float) * 0.25
    v = np.array([0.0, -2.0, 0.0])
    out = [oracle.el3d(var, xn, yn, zn, 0.07, 0.01, v, 1.0, True, 0.2)
           for var in (0, 1, 2)]
    for H, M, f in out[1:]:
        assert rel_l2(H, out[0][0]) < 1e-14
        assert rel_l2(M, out[0][1]) < 1e-13
        assert rel_l2(f, out[0][2]) < 1e-13


def test_ot_overflows_above_pe_709(oracle):
    xn = np.array([0, 1, 1, 0, 0, 1, 1, 0], float)
    yn = np.array([0, 0, 1, 1, 0, 0, 1, 1], float)
    zn = np.array([0, 0, 0, 0, 1, 1, 1, 1], float)
    v = np.array([1.0, 0.0, 0.0])
    # OT: h = 2/(1/1) = 2, Pe = |v| h / (2 lambda) = 1/lambda
    det, n, w, *_ = oracle.gauss_point(0, 0.1, 0.2, 0.3, xn, yn, zn,
                                       [1 / 800.0] * 3, v)
    assert np.isnan(w).all()
    det, n, w, *_ = oracle.gauss_point(0, 0.1, 0.2, 0.3, xn, yn, zn,
                                       [1 / 700.0] * 3, v)
    assert np.isfinite(w).all()
    det, n, w, *_ = oracle.gauss_point(2, 0.1, 0.2, 0.3, xn, yn, zn,
                                       [1 / 800.0] * 3, v)
    assert np.isfinite(w).all()


def test_vf_beta_branches_continuous(oracle):
    """VF's beta(Pe): series below 1e-3, 1 - 1/Pe above 50, tanh between;
    tau must be continuous across both switches."""
    xn = np.array([0, 1, 1, 0, 0, 1, 1, 0], float)
    yn = np.array([0, 0, 1, 1, 0, 0, 1, 1], float)
    zn = np.array([0, 0, 0, 0, 1, 1, 1, 1], float)
    v = np.array([1.0, 0.0, 0.0])

    def w_at(pe):  # VF: h = 1 -> Pe = 1/(2 lambda)
        lam = 1.0 / (2.0 * pe)
        return oracle.gauss_point(2, 0.1, 0.2, 0.3, xn, yn, zn, [lam] * 3, v)[2]

    for pe in (1e-3, 50.0):
        a, b = w_at(pe * (1 - 1e-9)), w_at(pe * (1 + 1e-9))
        assert np.max(np.abs(a - b)) < 1e-7


def test_bicg_and_bicgstab_agree(vdr, oracle):
    prob = vdr.problems.constant_advection(8, 8, 4, seed=3)
    m = prob.mesh
    bb, b, d = oracle.assemble(prob.variant, m.xx, m.yy, m.zz, m.iss,
                               prob.vel, prob.lam, prob.pdec, prob.q)
    b[prob.bc == 1] = 0
    d[prob.bc == 1] = 1
    x1, it1, e1, s1 = oracle.dbcg(b, np.zeros(m.nnode), bb, m.iss, d, prob.bc,
                                  1e-13, 5000)
    x2, it2, e2, s2 = oracle.bicgstab(b, np.zeros(m.nnode), bb, m.iss, d,
                                      prob.bc, 1e-13, 5000)
    assert s1 == 0 and s2 == 0
    assert rel_l2(x1, x2) < 1e-10


def test_openmp_apply_matches_serial(vdr, oracle):
    prob = vdr.problems.rotation_shear(10, 9, 7, seed=5)
    m = prob.mesh
    bb, _, _ = oracle.assemble(2, m.xx, m.yy, m.zz, m.iss, prob.vel, prob.lam,
                               prob.pdec, prob.q, nthreads=4)
    x = np.random.default_rng(4).standard_normal(m.nnode)
    c, nc = oracle.greedy_colors(m.iss, m.nnode)
    ce, co = oracle.color_lists(c, nc)
    for tr in (False, True):
        y, _ = oracle.matvec0(m.iss, bb, prob.bc, x, transpose=tr)
        y2 = oracle.matvec0_omp(m.iss, bb, prob.bc, ce, co, x, transpose=tr,
                                nthreads=4)
        assert rel_l2(y2, y) < 1e-14


def test_mesh_union_layout(vdr):
    """Concatenated meshes: node ids offset per mesh, every element inside
    its own node range, the cube sizes inside the drawn range."""
    P = vdr.problems
    sizes = P.cube_sizes(64, seed=2001, nmin=8, nmax=48)
    assert sizes.min() >= 8 and sizes.max() <= 48
    probs = P.cube_batch(5, seed=2001, nmin=2, nmax=5)
    u = P.concat(probs)
    m = u.mesh
    E = m.nelem
    assert E == sum(p.mesh.nelem for p in probs)
    assert m.nnode == sum(p.mesh.nnode for p in probs) == m.xx.size
    iss = m.iss.reshape(8, E).astype(np.int64) - 1
    seg = np.searchsorted(m.node_off, iss[0], side="right") - 1
    for k in range(8):
        assert np.all(iss[k] >= m.node_off[seg])
        assert np.all(iss[k] < m.node_off[seg + 1])
    for i, p in enumerate(probs):
        a, b = m.elem_off[i], m.elem_off[i + 1]
        assert np.array_equal(iss[:, a:b] - m.node_off[i],
                              p.mesh.iss.reshape(8, -1) - 1)
    assert u.bc.size == m.nnode and u.vel.size == 3 * E


def test_tilting_velocity_and_sources(vdr):
    """The learned workload's velocity: step 0 is the rotation_shear field,
    every step is scaled to max |u_e| = 1 and the axis tilts about y; the
    many-right-hand-side sources are seeded per column."""
    P = vdr.problems
    L = vdr.learned
    prob = P.rotation_shear(6, 5, 4, seed=7)
    v0 = L.tilted_velocity(prob.mesh, 0)
    assert np.allclose(v0, prob.vel, rtol=0, atol=1e-15)
    E = prob.mesh.nelem
    for step in (1, 40, 180):
        v = L.tilted_velocity(prob.mesh, step, tilt_deg=0.5).reshape(3, E)
        assert abs(np.sqrt((v * v).sum(axis=0)).max() - 1.0) < 1e-14
    # tilting 90 degrees puts the axis along x: no x component of rotation
    v90 = L.tilted_velocity(prob.mesh, 1, tilt_deg=90.0, shear=0.0).reshape(3, E)
    assert np.abs(v90[0]).max() < 1e-12
    Q1 = P.random_gaussian_sources(prob.mesh, 3, seed=3001)
    Q2 = P.random_gaussian_sources(prob.mesh, 3, seed=3001)
    assert np.array_equal(Q1, Q2) and not np.array_equal(Q1[0], Q1[1])
    assert np.array_equal(P.random_gaussian_sources(prob.mesh, 1, seed=3002)[0],
                          Q1[1])
