"""CPU oracle for the Vanadis EBE HEX8 directional-residual solve.

TEST INFRASTRUCTURE ONLY.  This package is the oracle: the test suite, the
smoke check and the CPU-baseline leg of the benchmark import it; the product
library (``libvdr.so`` and its Python host module) never does.  The numerics
live in ``vdr_oracle.c`` (a plain-C restatement of the reference's CPU build
``src_updates/vanadis_full_DR_OpenMP_timing.for``); this module loads it with
ctypes and adapts numpy arrays.

Parity pinning: the oracle reproduces the known-answer values of the
reference's only recorded run (``src_v2026_2_1/vanadis_log.txt``) and the
colour fixtures generated from the reference's own colouring functions; see
``tests/test_oracle_kat.py`` and ``tests/golden/``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libvdr_oracle.so")
_lib = None

DR_OT, DR_GP, DR_VF = 0, 1, 2
MASK_OT, MASK_VF = 0, 1

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_i = ctypes.c_int
_d = ctypes.c_double


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, seconds)."""
    src = os.path.join(_HERE, "vdr_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(src)):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        sigs = {
            "or_siatka": [_i, _i, _i, _D, _D, _D, _D, _D, _D],
            "or_w_el": [_i, _i, _i, _I],
            "or_kod_el_dr": [_i, _i, _i, _I],
            "or_build_bc_nodes": [_i, _i, _i, _I, _I, _i, _I],
            "or_gauss_point": [_i, _d, _d, _d, _D, _D, _D, _D, _D, _D, _D,
                               _D, _D, _D, _D],
            "or_el3d": [_i, _D, _D, _D, _d, _d, _D, _d, _i, _d, _D, _D, _D],
            "or_assemble": [_i, _i, _i, _D, _D, _D, _I, _I, _D, _D, _D, _D,
                            _d, _d, _d, _d, _d, _D, _D, _D, _D, _i],
            "or_matvec0": [_i, _i, _I, _D, _I, _D, _D],
            "or_mttvec0": [_i, _i, _I, _D, _I, _D, _D],
            "or_matvec0_omp": [_i, _i, _I, _D, _I, _I, _I, _i, _i, _D, _D,
                               _i],
            "or_dbcg": [_i, _i, _D, _D, _d, _i, _I, _D, _D, _I, _D, _I],
            "or_bicgstab": [_i, _i, _D, _D, _d, _i, _I, _D, _D, _I, _D, _I,
                            _I, _I, _i, _i],
            "or_dominance_factor": [_i, _i, _I, _D],
            "or_is_diag_dominant": [_i, _i, _I, _D],
            "or_integrate_mass": [_i, _I, _D, _D, _D, _D],
            "or_parity_colors": [_i, _i, _i, _I],
            "or_greedy_colors": [_i, _i, _I, _I],
            "or_color_lists": [_i, _I, _i, _I, _I],
        }
        for name, args in sigs.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = None
        for name in ("or_dbcg", "or_bicgstab", "or_is_diag_dominant",
                     "or_greedy_colors"):
            getattr(L, name).restype = _i
        for name in ("or_dominance_factor", "or_integrate_mass"):
            getattr(L, name).restype = _d
        _lib = L
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _ip(a):
    return None if a is None else a.ctypes.data_as(_I)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


# ---------------------------------------------------------------- mesh
def siatka(dx, dy, dz):
    dx, dy, dz = _f64(dx), _f64(dy), _f64(dz)
    n = len(dx) * len(dy) * len(dz)
    xx, yy, zz = (np.empty(n) for _ in range(3))
    lib().or_siatka(len(dx), len(dy), len(dz), _dp(dx), _dp(dy), _dp(dz),
                    _dp(xx), _dp(yy), _dp(zz))
    return xx, yy, zz


def w_el(nax, nay, naz):
    E = (nax - 1) * (nay - 1) * (naz - 1)
    iss = np.empty(8 * E, dtype=np.int32)
    lib().or_w_el(nax, nay, naz, _ip(iss))
    return iss


def kod_el_dr(nax, nay, naz):
    E = (nax - 1) * (nay - 1) * (naz - 1)
    kod = np.empty(6 * E, dtype=np.int32)
    lib().or_kod_el_dr(nax, nay, naz, _ip(kod))
    return kod


def build_bc_nodes(nax, nay, naz, iss, kod, mask_mode=MASK_VF):
    bc = np.empty(nax * nay * naz, dtype=np.int32)
    lib().or_build_bc_nodes(nax, nay, naz, _ip(_i32(iss)), _ip(_i32(kod)),
                            mask_mode, _ip(bc))
    return bc


# -------------------------------------------------------------- element
def gauss_point(variant, xi, eta, zeta, xn, yn, zn, lam3, v3):
    xn, yn, zn, lam3, v3 = map(_f64, (xn, yn, zn, lam3, v3))
    det = ctypes.c_double()
    out = [np.empty(8) for _ in range(5)]
    lib().or_gauss_point(variant, xi, eta, zeta, _dp(xn), _dp(yn), _dp(zn),
                         _dp(lam3), _dp(v3), ctypes.byref(det),
                         *[_dp(o) for o in out])
    n, w, dnx, dny, dnz = out
    return det.value, n, w, dnx, dny, dnz


def el3d(variant, xn, yn, zn, lam, pdec, v3, q, robin=False, alpha=0.0):
    xn, yn, zn, v3 = map(_f64, (xn, yn, zn, v3))
    H, M, f = np.empty(64), np.empty(64), np.empty(8)
    lib().or_el3d(variant, _dp(xn), _dp(yn), _dp(zn), lam, pdec, _dp(v3), q,
                  int(bool(robin)), alpha, _dp(H), _dp(M), _dp(f))
    return H.reshape(8, 8), M.reshape(8, 8), f


def assemble(variant, xx, yy, zz, iss, vel, lam, pdec=None, q=None,
             kod=None, robin_alpha=0.0, aH=1.0, aM=0.0, cf=1.0, rM=0.0,
             t_old=None, want_bb=True, want_b=True, want_diag=True,
             nthreads=1):
    """Element matrices BB = aH*H + aM*M, RHS and Jacobi diagonal."""
    xx, yy, zz, vel, lam, pdec, q, t_old = map(
        _f64, (xx, yy, zz, vel, lam, pdec, q, t_old))
    iss, kod = _i32(iss), _i32(kod)
    N, E = len(xx), len(lam)
    bb = np.empty(64 * E) if want_bb else None
    b = np.empty(N) if want_b else None
    diag = np.empty(N) if want_diag else None
    lib().or_assemble(variant, N, E, _dp(xx), _dp(yy), _dp(zz), _ip(iss),
                      _ip(kod), _dp(vel), _dp(lam), _dp(pdec), _dp(q),
                      robin_alpha, aH, aM, cf, rM, _dp(t_old), _dp(bb),
                      _dp(b), _dp(diag), nthreads)
    return bb, b, diag


# -------------------------------------------------------------- applies
def matvec0(iss, bb, bc, x, transpose=False):
    """y = P A P x (or P A^T P x).  Returns (y, x_masked)."""
    iss, bb, bc = _i32(iss), _f64(bb), _i32(bc)
    x = np.array(x, dtype=np.float64, copy=True)
    y = np.empty_like(x)
    fn = lib().or_mttvec0 if transpose else lib().or_matvec0
    fn(len(x), len(bb) // 64, _ip(iss), _dp(bb), _ip(bc), _dp(x), _dp(y))
    return y, x


def matvec0_omp(iss, bb, bc, color_elems, color_offsets, x, transpose=False,
                nthreads=None):
    iss, bb, bc = _i32(iss), _f64(bb), _i32(bc)
    ce, co = _i32(color_elems), _i32(color_offsets)
    x = np.array(x, dtype=np.float64, copy=True)
    y = np.empty_like(x)
    lib().or_matvec0_omp(len(x), len(bb) // 64, _ip(iss), _dp(bb), _ip(bc),
                         _ip(ce), _ip(co), len(co) - 1, int(transpose),
                         _dp(x), _dp(y), nthreads or os.cpu_count())
    return y


# -------------------------------------------------------------- solvers
def dbcg(b, x0, bb, iss, diag, bc, tol=1e-8, itmax=1000):
    b, bb, diag = _f64(b), _f64(bb), _f64(diag)
    iss, bc = _i32(iss), _i32(bc)
    x = np.array(x0, dtype=np.float64, copy=True)
    it, err = ctypes.c_int(), ctypes.c_double()
    st = lib().or_dbcg(len(b), len(bb) // 64, _dp(b), _dp(x), tol, itmax,
                       ctypes.byref(it), ctypes.byref(err), _dp(bb), _ip(iss),
                       _dp(diag), _ip(bc))
    return x, it.value, err.value, st


def bicgstab(b, x0, bb, iss, diag, bc, tol=1e-8, itmax=1000, colors=None,
             nthreads=1):
    b, bb, diag = _f64(b), _f64(bb), _f64(diag)
    iss, bc = _i32(iss), _i32(bc)
    x = np.array(x0, dtype=np.float64, copy=True)
    it, err = ctypes.c_int(), ctypes.c_double()
    ce = co = None
    nc = 0
    if colors is not None:
        ce, co = _i32(colors[0]), _i32(colors[1])
        nc = len(co) - 1
    st = lib().or_bicgstab(len(b), len(bb) // 64, _dp(b), _dp(x), tol, itmax,
                           ctypes.byref(it), ctypes.byref(err), _dp(bb),
                           _ip(iss), _dp(diag), _ip(bc), _ip(ce), _ip(co), nc,
                           nthreads)
    return x, it.value, err.value, st


# ---------------------------------------------------------- diagnostics
def dominance_factor(iss, bb, nnode):
    return lib().or_dominance_factor(nnode, len(bb) // 64, _ip(_i32(iss)),
                                     _dp(_f64(bb)))


def is_diag_dominant(iss, bb, nnode):
    return bool(lib().or_is_diag_dominant(nnode, len(bb) // 64,
                                          _ip(_i32(iss)), _dp(_f64(bb))))


def integrate_mass(iss, xx, yy, zz, c):
    iss = _i32(iss)
    return lib().or_integrate_mass(len(iss) // 8, _ip(iss), _dp(_f64(xx)),
                                   _dp(_f64(yy)), _dp(_f64(zz)),
                                   _dp(_f64(c)))


# ------------------------------------------------------------ colouring
def parity_colors(nax, nay, naz):
    E = (nax - 1) * (nay - 1) * (naz - 1)
    c = np.empty(E, dtype=np.int32)
    lib().or_parity_colors(nax, nay, naz, _ip(c))
    return c


def greedy_colors(iss, nnode):
    iss = _i32(iss)
    c = np.empty(len(iss) // 8, dtype=np.int32)
    nc = lib().or_greedy_colors(nnode, len(c), _ip(iss), _ip(c))
    return c, nc


def color_lists(color, ncolors):
    color = _i32(color)
    ce = np.empty(len(color), dtype=np.int32)
    co = np.empty(ncolors + 1, dtype=np.int32)
    lib().or_color_lists(len(color), _ip(color), ncolors, _ip(ce), _ip(co))
    return ce, co
