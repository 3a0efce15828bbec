"""Seeded synthetic problems for the EBE HEX8 DR solve.

The reference ships one recorded case (a 7x20x20 node mesh); the larger
workloads are synthetic stand-ins with the shapes, sizes and value
distributions of the benchmark configurations, built here from a
counter-based SplitMix64 generator so that every host (x86 or Arm) produces
bit-identical inputs.  Layouts follow the reference driver:

* node numbering ``n = i + nax*j + nax*nay*k`` (x fastest), as ``siatka``
  (vanadis_full_DR_OpenMP_timing.for:201-219);
* element connectivity ``iss(E,8)`` column-major, 1-based, local node order
  (0,0,0),(1,0,0),(1,1,0),(0,1,0),(0,0,1),(1,0,1),(1,1,1),(0,1,1), elements
  x fastest, as ``w_el`` (:221-251);
* face codes ``kod(E,6)`` as ``kod_el_dr`` (:253-295);
* per-element fields evaluated at the element centroid: velocity ``(E,3)``
  column-major, isotropic diffusivity, decay rate and source (kg/s), i.e.
  the values the reference's per-element hook ``atmosfera`` (:163-199)
  returns for element ``nr_el``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

DR_OT, DR_GP, DR_VF = 0, 1, 2

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    """n uniforms in [0,1) for (seed, stream), counter-based."""
    with np.errstate(over="ignore"):
        key = _splitmix64(np.array([(seed << 20) ^ stream], dtype=np.uint64))[0]
        ctr = np.arange(n, dtype=np.uint64) + key
    z = _splitmix64(ctr)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    """Standard normals by Box-Muller from two uniform streams."""
    u1 = uniform(seed, stream, n)
    u2 = uniform(seed, stream + 1, n)
    return np.sqrt(-2.0 * np.log1p(-u1)) * np.cos(2.0 * math.pi * u2)


@dataclass
class Mesh:
    nax: int
    nay: int
    naz: int
    xx: np.ndarray
    yy: np.ndarray
    zz: np.ndarray
    iss: np.ndarray  # int32 [8*E], column-major (E,8), 1-based
    kod: np.ndarray  # int32 [6*E], column-major (E,6)

    @property
    def nnode(self) -> int:
        return self.nax * self.nay * self.naz

    @property
    def nelem(self) -> int:
        return (self.nax - 1) * (self.nay - 1) * (self.naz - 1)


@dataclass
class MeshUnion(Mesh):
    """Several meshes side by side (no element couples two of them): node
    ids of mesh m are offset by node_off[m], elements concatenated."""
    n_node: int = 0
    n_elem: int = 0
    node_off: np.ndarray = None
    elem_off: np.ndarray = None

    @property
    def nnode(self) -> int:
        return self.n_node

    @property
    def nelem(self) -> int:
        return self.n_elem


@dataclass
class Problem:
    name: str
    mesh: Mesh
    vel: np.ndarray  # [3*E] column-major
    lam: np.ndarray
    pdec: np.ndarray
    q: np.ndarray
    bc: np.ndarray  # int32 [N]
    robin_alpha: float = 0.0
    variant: int = DR_VF
    tol: float = 1e-8
    meta: dict = field(default_factory=dict)


def connectivity(nax: int, nay: int, naz: int) -> np.ndarray:
    """iss(E,8), column-major, 1-based; same numbers as w_el."""
    nex, ney, nez = nax - 1, nay - 1, naz - 1
    k, j, i = np.meshgrid(np.arange(nez), np.arange(ney), np.arange(nex),
                          indexing="ij")
    base = (i + nax * j + nax * nay * k).ravel().astype(np.int64) + 1
    pl = nax * nay
    offs = [0, 1, 1 + nax, nax, pl, 1 + pl, 1 + pl + nax, pl + nax]
    iss = np.concatenate([base + o for o in offs])
    return iss.astype(np.int32)


def face_codes(nax: int, nay: int, naz: int) -> np.ndarray:
    """kod(E,6), column-major; same numbers as kod_el_dr."""
    nex, ney, nez = nax - 1, nay - 1, naz - 1
    k, j, i = np.meshgrid(np.arange(nez), np.arange(ney), np.arange(nex),
                          indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    kod = np.zeros((6, i.size), dtype=np.int32)
    kod[0][k == 0] = 1
    kod[1][k == nez - 1] = 2
    kod[2][i == 0] = 3
    kod[3][i == nex - 1] = 4
    kod[4][j == ney - 1] = 5
    kod[5][j == 0] = 6
    return kod.ravel()


MASK_OT, MASK_VF = 0, 1


def face_dirichlet(mesh: Mesh, mode: int = MASK_VF) -> np.ndarray:
    """The reference's Dirichlet node mask from face codes: the nodes of
    faces 1,2,4,5,6 of every element carrying that code (face 3 is the
    Robin face).  MASK_VF follows src_v2026_2_1/VANADIS.FOR:2026-2110;
    MASK_OT follows vanadis_full_DR_OpenMP_timing.for:1719-1810, whose face
    5/6 node lists mark the interior node rows y=1 and y=nay-2."""
    E = mesh.nelem
    iss = mesh.iss.reshape(8, E).astype(np.int64) - 1
    kod = mesh.kod.reshape(6, E)
    lo, hi = (0, 1, 5, 4), (3, 2, 6, 7)
    faces = {1: (0, 1, 2, 3), 2: (4, 5, 6, 7), 4: (1, 2, 6, 5),
             5: lo if mode == MASK_OT else hi,
             6: hi if mode == MASK_OT else lo}
    bc = np.zeros(mesh.nnode, dtype=np.int32)
    for f, loc in faces.items():
        sel = kod[f - 1] == f
        for s in loc:
            bc[iss[s][sel]] = 1
    return bc


def structured_mesh(nex: int, ney: int, nez: int, jitter: float = 0.0,
                    seed: int = 0, lengths=(1.0, 1.0, 1.0)) -> Mesh:
    """Unit-box HEX8 mesh; interior coordinates jittered uniformly by up to
    +-jitter of the local spacing (boundary coordinates stay on the box)."""
    nax, nay, naz = nex + 1, ney + 1, nez + 1
    gx = np.linspace(0.0, lengths[0], nax)
    gy = np.linspace(0.0, lengths[1], nay)
    gz = np.linspace(0.0, lengths[2], naz)
    zz, yy, xx = np.meshgrid(gz, gy, gx, indexing="ij")
    xx, yy, zz = xx.ravel().copy(), yy.ravel().copy(), zz.ravel().copy()
    if jitter > 0.0:
        n = xx.size
        kk, jj, ii = np.meshgrid(np.arange(naz), np.arange(nay),
                                 np.arange(nax), indexing="ij")
        ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()
        for arr, idx, nmax, h, stream in (
                (xx, ii, nax - 1, lengths[0] / nex, 1),
                (yy, jj, nay - 1, lengths[1] / ney, 3),
                (zz, kk, naz - 1, lengths[2] / nez, 5)):
            u = uniform(seed, stream, n)
            inner = (idx > 0) & (idx < nmax)
            arr[inner] += (2.0 * u[inner] - 1.0) * jitter * h
    return Mesh(nax, nay, naz, xx, yy, zz, connectivity(nax, nay, naz),
                face_codes(nax, nay, naz))


def axis_mesh(dx, dy, dz) -> Mesh:
    """Tensor-product mesh from axis coordinate lists (siatka,
    vanadis_full_DR_OpenMP_timing.for:201-219)."""
    dx, dy, dz = (np.asarray(a, dtype=np.float64) for a in (dx, dy, dz))
    nax, nay, naz = len(dx), len(dy), len(dz)
    zz, yy, xx = np.meshgrid(dz, dy, dx, indexing="ij")
    return Mesh(nax, nay, naz, xx.ravel().copy(), yy.ravel().copy(),
                zz.ravel().copy(), connectivity(nax, nay, naz),
                face_codes(nax, nay, naz))


def uniform_fields_problem(name, mesh: Mesh, lam, pdec, vel3, q_total=0.0,
                           source_element=None, robin_alpha=0.0,
                           mask_mode=MASK_VF, variant=DR_VF,
                           tol=1e-8) -> Problem:
    """Constant fields as the reference's configuration file sets them
    (atmosfera, vanadis_full_DR_OpenMP_timing.for:163-199): one diffusivity,
    decay rate and velocity for all elements, the whole source q_total in
    one element (1-based id, as nr_el), Robin coefficient on face 3, and the
    face-code Dirichlet mask."""
    E = mesh.nelem
    vel = np.concatenate([np.full(E, float(v)) for v in vel3])
    q = np.zeros(E)
    if source_element is not None:
        q[source_element - 1] = q_total
    return Problem(name, mesh, vel, np.full(E, float(lam)),
                   np.full(E, float(pdec)), q, face_dirichlet(mesh, mask_mode),
                   float(robin_alpha), variant, tol)


def centroids(mesh: Mesh):
    E = mesh.nelem
    nd = mesh.iss.reshape(8, E).astype(np.int64) - 1
    cx = mesh.xx[nd].mean(axis=0)
    cy = mesh.yy[nd].mean(axis=0)
    cz = mesh.zz[nd].mean(axis=0)
    return cx, cy, cz


def inflow_mask(mesh: Mesh, vel: np.ndarray) -> np.ndarray:
    """Dirichlet nodes: the 4 nodes of every boundary face whose element
    velocity points into the domain (u_e . n_out < 0)."""
    nax, nay, naz = mesh.nax, mesh.nay, mesh.naz
    nex, ney, nez = nax - 1, nay - 1, naz - 1
    E = mesh.nelem
    u = vel.reshape(3, E)
    k, j, i = np.meshgrid(np.arange(nez), np.arange(ney), np.arange(nex),
                          indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    bc = np.zeros(mesh.nnode, dtype=np.int32)

    def mark(sel, fixed_axis, fixed_val):
        ii, jj, kk = i[sel], j[sel], k[sel]
        for da in (0, 1):
            for db in (0, 1):
                if fixed_axis == 0:
                    n = fixed_val + nax * (jj + da) + nax * nay * (kk + db)
                elif fixed_axis == 1:
                    n = (ii + da) + nax * fixed_val + nax * nay * (kk + db)
                else:
                    n = (ii + da) + nax * (jj + db) + nax * nay * fixed_val
                bc[n] = 1

    mark((i == 0) & (u[0] > 0), 0, 0)
    mark((i == nex - 1) & (u[0] < 0), 0, nex)
    mark((j == 0) & (u[1] > 0), 1, 0)
    mark((j == ney - 1) & (u[1] < 0), 1, ney)
    mark((k == 0) & (u[2] > 0), 2, 0)
    mark((k == nez - 1) & (u[2] < 0), 2, nez)
    return bc


def _gauss_sources(cx, cy, cz, centres, sigma, cell_volume):
    g = np.zeros_like(cx)
    for (x0, y0, z0), s in zip(centres, sigma):
        r2 = (cx - x0) ** 2 + (cy - y0) ** 2 + (cz - z0) ** 2
        g += np.exp(-r2 / (2.0 * s * s))
    return g * cell_volume


def random_gaussian_sources(mesh: Mesh, K: int, seed: int = 3001,
                            cell_volume: float | None = None) -> np.ndarray:
    """K per-element source fields (K x E): source k is one Gaussian blob,
    seeded by seed + k, with centre uniform in [0.1, 0.9]^3 and sigma
    uniform in [0.03, 0.1] -- the right-hand sides of the batched
    many-right-hand-side workload."""
    cx, cy, cz = centroids(mesh)
    if cell_volume is None:
        cell_volume = 1.0 / mesh.nelem
    Q = np.empty((K, mesh.nelem))
    for k in range(K):
        u = uniform(seed + k, 21, 4)
        centre = tuple(0.1 + 0.8 * u[:3])
        Q[k] = _gauss_sources(cx, cy, cz, [centre], [0.03 + 0.07 * u[3]],
                              cell_volume)
    return Q


def rotation_cube(n: int, seed: int, variant=DR_VF) -> Problem:
    """One mesh of the many-mesh workload: n^3 elements on the jittered
    unit cube, solid-body rotation about a seeded random axis through the
    centre scaled to max |u_e| = 1, lognormal diffusivity exp(ln 1e-4 + xi),
    one Gaussian source (seeded centre in [0.2, 0.8]^3, sigma in
    [0.05, 0.1]), zero Dirichlet on inflow faces, tolerance 1e-8."""
    mesh = structured_mesh(n, n, n, 0.1, seed)
    E = mesh.nelem
    cx, cy, cz = centroids(mesh)
    g = normal(seed, 31, 3)
    ax = g / np.linalg.norm(g)
    rx, ry, rz = cx - 0.5, cy - 0.5, cz - 0.5
    ux = ax[1] * rz - ax[2] * ry
    uy = ax[2] * rx - ax[0] * rz
    uz = ax[0] * ry - ax[1] * rx
    sc = 1.0 / np.sqrt(ux * ux + uy * uy + uz * uz).max()
    vel = np.concatenate([ux * sc, uy * sc, uz * sc])
    lam = np.exp(math.log(1e-4) + normal(seed, 11, E))
    u = uniform(seed, 33, 4)
    q = _gauss_sources(cx, cy, cz, [tuple(0.2 + 0.6 * u[:3])],
                       [0.05 + 0.05 * u[3]], 1.0 / E)
    return Problem("rotation_cube_%d" % n, mesh, vel, lam, np.zeros(E), q,
                   inflow_mask(mesh, vel), 0.0, variant, 1e-8, {"seed": seed})


def cube_sizes(nmesh: int = 256, seed: int = 2001, nmin: int = 8,
               nmax: int = 48) -> np.ndarray:
    """Cube edges (elements) drawn uniformly from nmin..nmax."""
    u = uniform(seed, 41, nmesh)
    return (nmin + np.floor(u * (nmax - nmin + 1))).astype(int)


def cube_batch(nmesh: int = 256, seed: int = 2001, nmin: int = 8,
               nmax: int = 48) -> list:
    """The many-mesh workload: mesh m is rotation_cube(n_m, seed + m)."""
    return [rotation_cube(int(n), seed + m)
            for m, n in enumerate(cube_sizes(nmesh, seed, nmin, nmax))]


def concat(problems: list) -> Problem:
    """One problem holding several meshes side by side (the block-diagonal
    system of all of them); its mesh records node_off / elem_off."""
    Ns = [p.mesh.nnode for p in problems]
    Es = [p.mesh.nelem for p in problems]
    node_off = np.concatenate([[0], np.cumsum(Ns)]).astype(np.int64)
    elem_off = np.concatenate([[0], np.cumsum(Es)]).astype(np.int64)
    iss = np.concatenate(
        [p.mesh.iss.reshape(8, E).astype(np.int64) + o
         for p, E, o in zip(problems, Es, node_off[:-1])], axis=1)
    kod = np.concatenate([p.mesh.kod.reshape(6, E)
                          for p, E in zip(problems, Es)], axis=1)
    vel = np.concatenate([p.vel.reshape(3, E) for p, E in zip(problems, Es)],
                         axis=1)
    mesh = MeshUnion(0, 0, 0,
                     np.concatenate([p.mesh.xx for p in problems]),
                     np.concatenate([p.mesh.yy for p in problems]),
                     np.concatenate([p.mesh.zz for p in problems]),
                     iss.astype(np.int32).ravel(), kod.astype(np.int32).ravel(),
                     n_node=int(node_off[-1]), n_elem=int(elem_off[-1]),
                     node_off=node_off, elem_off=elem_off)
    return Problem("union_of_%d" % len(problems), mesh, vel.ravel(),
                   np.concatenate([p.lam for p in problems]),
                   np.concatenate([p.pdec for p in problems]),
                   np.concatenate([p.q for p in problems]),
                   np.concatenate([p.bc for p in problems]),
                   problems[0].robin_alpha, problems[0].variant,
                   problems[0].tol, {"meshes": len(problems)})


def constant_advection(nex=32, ney=32, nez=16, seed=1001) -> Problem:
    """Small FP64 case: constant velocity (1,0.5,0.25)/|.|, diffusivity
    1e-3, Gaussian source (sigma 0.08) at (0.3,0.5,0.5), zero Dirichlet on
    inflow faces, OT DR variant, tolerance 1e-10."""
    mesh = structured_mesh(nex, ney, nez, 0.1, seed)
    E = mesh.nelem
    v = np.array([1.0, 0.5, 0.25])
    v = v / np.linalg.norm(v)
    vel = np.concatenate([np.full(E, v[0]), np.full(E, v[1]),
                          np.full(E, v[2])])
    cx, cy, cz = centroids(mesh)
    q = _gauss_sources(cx, cy, cz, [(0.3, 0.5, 0.5)], [0.08],
                       1.0 / (nex * ney * nez))
    return Problem("constant_advection_%dx%dx%d" % (nex, ney, nez), mesh, vel,
                   np.full(E, 1e-3), np.zeros(E), q, inflow_mask(mesh, vel),
                   0.0, DR_OT, 1e-10, {"seed": seed})


ROTATION_SOURCES = [(0.3, 0.5, 0.3), (0.7, 0.4, 0.6)]


def rotation_shear(nex=256, ney=256, nez=128, seed=1002,
                   variant=DR_VF) -> Problem:
    """Large FP64 case: solid-body rotation about the z axis through
    (0.5,0.5) plus shear u_x += 0.3 z, scaled to max |u_e| = 1; lognormal
    diffusivity exp(ln 1e-4 + xi), xi ~ N(0,1) per element; two Gaussian
    sources (sigma 0.05) at ROTATION_SOURCES; zero Dirichlet on inflow
    faces; tolerance 1e-8.  The VF (numerically safe) DR variant is the
    default because the OT variant's exp-based coth overflows for Pe > 709,
    which the lognormal tail reaches."""
    mesh = structured_mesh(nex, ney, nez, 0.1, seed)
    E = mesh.nelem
    cx, cy, cz = centroids(mesh)
    ux = -(cy - 0.5) + 0.3 * cz
    uy = cx - 0.5
    uz = np.zeros(E)
    s = 1.0 / np.sqrt(ux * ux + uy * uy + uz * uz).max()
    vel = np.concatenate([ux * s, uy * s, uz * s])
    lam = np.exp(math.log(1e-4) + normal(seed, 11, E))
    q = _gauss_sources(cx, cy, cz, ROTATION_SOURCES, [0.05, 0.05],
                       1.0 / (nex * ney * nez))
    return Problem("rotation_shear_%dx%dx%d" % (nex, ney, nez), mesh, vel,
                   lam, np.zeros(E), q, inflow_mask(mesh, vel), 0.0, variant,
                   1e-8, {"seed": seed})
