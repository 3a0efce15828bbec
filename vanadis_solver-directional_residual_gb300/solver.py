"""Host-side mirror of the reference's solve interface over libvdr.so.

* ``kernel_dbcg_simple(...)`` -- the reference's entry point
  (src_v2026_2_1/cudatest.cu:301-305, called from VANADIS.FOR:809-810) with
  its argument meaning: stored element matrices BB, ISS(E,8), DIAG, node
  counts and the Dirichlet mask in; X, ITER, ERR out.
* ``Solver`` -- the handle API: mesh and per-element fields stay resident
  on the GPU, the DR element terms are recomputed there, and the solve,
  apply, right-hand-side assembly and mass integral run on device.

Host arrays are numpy; device arrays may be any object exposing
``data_ptr()`` (torch CUDA tensors), which the ``*_device`` methods use
without copies.
"""
from __future__ import annotations

import ctypes
import functools
import sys
from dataclasses import dataclass

import numpy as np

from . import _lib as L

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _ip(a):
    return None if a is None else a.ctypes.data_as(_I)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


def _ptr(t):
    return None if t is None else ctypes.c_void_p(int(t.data_ptr()))


def _stream_order(owner):
    """(torch current stream, the library stream as a torch stream) when
    torch has initialised CUDA, else None.  The handle's stream is
    non-blocking, so device arrays written by torch must be ordered before
    a library call and torch's later work after it."""
    torch = sys.modules.get("torch")
    if torch is None or not torch.cuda.is_initialized():
        return None
    if owner._ext_stream is None:
        owner._ext_stream = torch.cuda.ExternalStream(owner.stream())
    cur = torch.cuda.current_stream()
    if cur.cuda_stream == owner._ext_stream.cuda_stream:
        return None
    return cur, owner._ext_stream


def _device_call(fn):
    """Orders a device-array call between torch's current stream and the
    library's stream (events, no host synchronisation)."""
    @functools.wraps(fn)
    def wrapper(self, *args, **kwargs):
        owner = getattr(self, "solver", self)
        so = _stream_order(owner)
        if so:
            so[1].wait_stream(so[0])
        try:
            return fn(self, *args, **kwargs)
        finally:
            if so:
                so[0].wait_stream(so[1])
    return wrapper


_VARIANTS = {"ot": L.DR_OT, "gp": L.DR_GP, "vf": L.DR_VF}
_SCATTER = {"auto": L.SCATTER_AUTO, "atomic": L.SCATTER_ATOMIC,
            "color": L.SCATTER_COLOR, "colour": L.SCATTER_COLOR,
            "warp": L.SCATTER_WARP}
_APPLY = {"auto": L.APPLY_AUTO, "stored": L.APPLY_STORED,
          "matrix_free": L.APPLY_MATRIX_FREE}
_SOLVER = {"bicgstab": L.SOLVER_BICGSTAB, "bicg": L.SOLVER_BICG}
_STORE = {"auto": L.STORE_AUTO, "fp64": L.STORE_FP64, "df": L.STORE_DF}


@dataclass
class Options:
    dr_variant: object = None  # None -> the problem's; or "ot"/"gp"/"vf"/int
    scatter: str = "auto"
    apply_mode: str = "auto"
    solver: str = "bicgstab"
    iters_per_graph: int = 8
    device: int = 0
    matrix_storage: str = "auto"
    precision: str = "fp64"      # "fp64" or "mixed" (FP64 refinement, FP32 inner)

    def to_c(self, default_variant: int) -> L.VdrOptions:
        o = L.VdrOptions()
        L.load_library().vdr_default_options(ctypes.byref(o))
        v = self.dr_variant
        if v is None:
            v = default_variant
        o.dr_variant = _VARIANTS[v] if isinstance(v, str) else int(v)
        o.scatter = _SCATTER[self.scatter]
        o.apply_mode = _APPLY[self.apply_mode]
        o.solver = _SOLVER[self.solver]
        o.iters_per_graph = int(self.iters_per_graph)
        o.device = int(self.device)
        o.matrix_storage = _STORE[self.matrix_storage]
        o.precision = {"fp64": L.PRECISION_FP64, "mixed": L.PRECISION_MIXED}[self.precision]
        return o


class Solver:
    """GPU-resident EBE DR operator and Krylov solver for one mesh."""

    def __init__(self, problem, options: Options | None = None,
                 aH: float = 1.0, aM: float = 0.0):
        self._ext_stream = None
        self.lib = L.load_library()
        self.problem = problem
        self.options = options or Options()
        m = problem.mesh
        self.N, self.E = m.nnode, m.nelem
        self._keep = [_f64(m.xx), _f64(m.yy), _f64(m.zz), _i32(m.iss),
                      _i32(m.kod)]
        xx, yy, zz, iss, kod = self._keep
        h = ctypes.c_void_p()
        opt = self.options.to_c(problem.variant)
        L.check(self.lib.vdr_create(ctypes.byref(h), self.N, self.E, _dp(xx),
                                    _dp(yy), _dp(zz), _ip(iss), _ip(kod),
                                    ctypes.byref(opt)), "vdr_create")
        self.h = h
        self.set_fields(problem.vel, problem.lam, problem.pdec, problem.q,
                        problem.robin_alpha)
        self.set_dirichlet(problem.bc)
        self.set_operator(aH, aM)

    # -- configuration -------------------------------------------------
    def set_fields(self, vel, lam, pdec=None, q=None, robin_alpha=0.0):
        L.check(self.lib.vdr_set_fields(self.h, _dp(_f64(vel)), _dp(_f64(lam)),
                                        _dp(_f64(pdec)), _dp(_f64(q)),
                                        float(robin_alpha)), "vdr_set_fields")

    def set_dirichlet(self, bc):
        L.check(self.lib.vdr_set_dirichlet(self.h, _ip(_i32(bc))),
                "vdr_set_dirichlet")

    def set_operator(self, aH: float, aM: float):
        L.check(self.lib.vdr_set_operator(self.h, float(aH), float(aM)),
                "vdr_set_operator")

    # -- host-array calls ---------------------------------------------
    def apply(self, x, transpose=False):
        x = _f64(x)
        y = np.empty(self.N)
        L.check(self.lib.vdr_apply(self.h, _dp(x), _dp(y), int(transpose)),
                "vdr_apply")
        return y

    def assemble_rhs(self, cf=1.0, rM=0.0, t_old=None, out=None):
        """Right-hand side into a new array, or into `out` (float64, N;
        pinned host memory makes the copy a DMA)."""
        b = np.empty(self.N) if out is None else out
        L.check(self.lib.vdr_assemble_rhs(self.h, float(cf), float(rM),
                                          _dp(_f64(t_old)), _dp(b)),
                "vdr_assemble_rhs")
        return b

    def diag(self):
        d = np.empty(self.N)
        L.check(self.lib.vdr_get_diag(self.h, _dp(d)), "vdr_get_diag")
        return d

    def element_matrices(self, out=None):
        """The operator's element matrices in the reference's BB layout
        (64 E float64, bb[64e + 8i + j] = A_e(i, j)): what
        kernel_dbcg_simple takes as BB.  `out` may be pinned host memory."""
        bb = np.empty(64 * self.problem.mesh.nelem) if out is None else out
        L.check(self.lib.vdr_get_element_matrices(self.h, _dp(bb)),
                "vdr_get_element_matrices")
        return bb

    def solve(self, b, x0=None, tol=None, itmax=1000, out=None):
        """Returns (x, iterations, relative residual, status).  With `out`
        (float64, N) the solution is written there, starting from x0 (or
        from out's own contents when x0 is None)."""
        b = _f64(b)
        if out is not None:
            x = out
            if x0 is not None and x0 is not out:
                x[:] = x0
        else:
            x = np.zeros(self.N) if x0 is None else np.array(x0, dtype=np.float64)
        it, err = ctypes.c_int(0), ctypes.c_double(0.0)
        tol = self.problem.tol if tol is None else tol
        st = self.lib.vdr_solve(self.h, _dp(b), _dp(x), float(tol), int(itmax),
                                ctypes.byref(it), ctypes.byref(err))
        L.check(st, "vdr_solve", allow=(L.OK, L.NOT_CONVERGED, L.BREAKDOWN))
        return x, it.value, err.value, st

    def mass(self, c):
        m = ctypes.c_double()
        L.check(self.lib.vdr_mass(self.h, _dp(_f64(c)), ctypes.byref(m)),
                "vdr_mass")
        return m.value

    # -- device-array calls (torch CUDA tensors or anything with data_ptr)
    @_device_call
    def apply_device(self, x, y, transpose=False):
        L.check(self.lib.vdr_apply_device(self.h, _ptr(x), _ptr(y),
                                          int(transpose)), "vdr_apply_device")

    @_device_call
    def apply_accumulate_device(self, x, y, transpose=False):
        L.check(self.lib.vdr_apply_accumulate_device(self.h, _ptr(x), _ptr(y),
                                                     int(transpose)),
                "vdr_apply_accumulate_device")

    @_device_call
    def apply32_device(self, x, y, transpose=False):
        """y = P A32 P x with the FP32 operator."""
        L.check(self.lib.vdr_apply32_device(self.h, _ptr(x), _ptr(y),
                                            int(transpose)), "vdr_apply32_device")

    @_device_call
    def assemble_rhs_device(self, b, cf=1.0, rM=0.0, t_old=None):
        L.check(self.lib.vdr_assemble_rhs_device(self.h, float(cf), float(rM),
                                                 _ptr(t_old), _ptr(b)),
                "vdr_assemble_rhs_device")

    @_device_call
    def solve_device(self, b, x, tol=None, itmax=1000):
        it, err = ctypes.c_int(0), ctypes.c_double(0.0)
        tol = self.problem.tol if tol is None else tol
        st = self.lib.vdr_solve_device(self.h, _ptr(b), _ptr(x), float(tol),
                                       int(itmax), ctypes.byref(it),
                                       ctypes.byref(err))
        L.check(st, "vdr_solve_device",
                allow=(L.OK, L.NOT_CONVERGED, L.BREAKDOWN))
        return it.value, err.value, st

    def set_segments(self, node_off):
        """Declare independent meshes: node ranges [off[m], off[m+1])."""
        off = _i32(node_off)
        L.check(self.lib.vdr_set_segments(self.h, int(off.size - 1), _ip(off)),
                "vdr_set_segments")
        self.nseg = int(off.size - 1)

    @_device_call
    def solve_segmented_device(self, b, x, tol=None, itmax=1000):
        """All meshes at once, per-mesh convergence.  Returns (iterations,
        relative residuals, statuses) per mesh and the overall status."""
        n = self.nseg
        its = np.zeros(n, dtype=np.int32)
        errs = np.zeros(n)
        sts = np.zeros(n, dtype=np.int32)
        tol = self.problem.tol if tol is None else tol
        st = self.lib.vdr_solve_segmented_device(self.h, _ptr(b), _ptr(x),
                                                 float(tol), int(itmax), _ip(its),
                                                 _dp(errs), _ip(sts))
        L.check(st, "vdr_solve_segmented_device",
                allow=(L.OK, L.NOT_CONVERGED, L.BREAKDOWN))
        return its, errs, sts, st

    def segment_tuning(self):
        t, th = ctypes.c_int(0), ctypes.c_int(0)
        L.check(self.lib.vdr_segment_tuning(self.h, ctypes.byref(t),
                                            ctypes.byref(th)),
                "vdr_segment_tuning")
        return t.value, th.value

    def apply_tuning(self) -> dict:
        """The applies' launch shapes chosen by measurement
        (vdr_apply_tuning): blocks per SM of the stored and binary16 applies
        with the time per apply of each candidate, and the block apply's box
        height and column halves with the times of (2,2), (2,1), (4,2) and
        of the tcgen05 box apply, and whether that one was chosen."""
        t = L.VdrApplyTuning()
        L.check(self.lib.vdr_apply_tuning(self.h, ctypes.byref(t)), "vdr_apply_tuning")
        grid = list(t.grid_candidates)
        return {"apply_blocks_per_sm": t.apply_blocks_per_sm,
                "apply_ms": dict(zip(grid, [round(v, 4) for v in t.apply_ms])),
                "half_blocks_per_sm": t.half_blocks_per_sm,
                "half_ms": dict(zip(grid, [round(v, 4) for v in t.half_ms])),
                "block_tile_y": t.block_tile_y, "block_halves": t.block_halves,
                "block_ms": dict(zip(["2x2", "2x1", "4x2", "tcgen05"],
                                     [round(v, 4) for v in t.block_ms])),
                "block_tcgen05": bool(t.block_tcgen05)}

    @_device_call
    def solve_learned_device(self, net, b, x, tol=None, itmax=1000,
                             stall_window=20):
        """Flexible BiCGStab right-preconditioned by the learned network
        (Jacobi-BiCGStab takes over on a stall).  Returns (iterations,
        relative residual, status, fell_back)."""
        it, err, fb = ctypes.c_int(0), ctypes.c_double(0.0), ctypes.c_int(0)
        tol = self.problem.tol if tol is None else tol
        st = self.lib.vdr_solve_learned_device(
            self.h, net.h, _ptr(b), _ptr(x), float(tol), int(itmax),
            int(stall_window), ctypes.byref(it), ctypes.byref(err),
            ctypes.byref(fb))
        L.check(st, "vdr_solve_learned_device",
                allow=(L.OK, L.NOT_CONVERGED, L.BREAKDOWN))
        return it.value, err.value, st, bool(fb.value)

    @_device_call
    def solve_gcr_device(self, b, x, net=None, tol=None, itmax=1000,
                         restart=20, stall_window=0):
        """Restarted GCR (flexible minimal residual) with Jacobi, or with
        the learned network as right preconditioner (Jacobi-BiCGStab takes
        over on a stall).  Returns (iterations, relative residual, status,
        fell_back)."""
        it, err, fb = ctypes.c_int(0), ctypes.c_double(0.0), ctypes.c_int(0)
        tol = self.problem.tol if tol is None else tol
        st = self.lib.vdr_solve_gcr_device(
            self.h, net.h if net is not None else None, _ptr(b), _ptr(x),
            float(tol), int(itmax), int(restart), int(stall_window),
            ctypes.byref(it), ctypes.byref(err), ctypes.byref(fb))
        L.check(st, "vdr_solve_gcr_device",
                allow=(L.OK, L.NOT_CONVERGED, L.BREAKDOWN))
        return it.value, err.value, st, bool(fb.value)

    @_device_call
    def solve_learned_hybrid_device(self, net, b, x, tol=None, itmax=1000,
                                    learned_steps=2):
        """learned_steps GCR steps with the network, then Jacobi-BiCGStab.
        Returns (iterations, relative residual, status, False)."""
        it, err = ctypes.c_int(0), ctypes.c_double(0.0)
        tol = self.problem.tol if tol is None else tol
        st = self.lib.vdr_solve_learned_hybrid_device(
            self.h, net.h, _ptr(b), _ptr(x), float(tol), int(itmax),
            int(learned_steps), ctypes.byref(it), ctypes.byref(err))
        L.check(st, "vdr_solve_learned_hybrid_device",
                allow=(L.OK, L.NOT_CONVERGED, L.BREAKDOWN))
        return it.value, err.value, st, False

    @_device_call
    def solve_gcr_record_device(self, b, x, hist, net=None, tol=None,
                                itmax=1000, restart=20):
        """GCR recording every iterate into hist.  Returns (recorded,
        iterations, relative residual, status)."""
        it, err, nh = ctypes.c_int(0), ctypes.c_double(0.0), ctypes.c_int(0)
        tol = self.problem.tol if tol is None else tol
        st = self.lib.vdr_solve_gcr_record_device(
            self.h, net.h if net is not None else None, _ptr(b), _ptr(x),
            float(tol), int(itmax), int(restart), _ptr(hist),
            int(hist.shape[0]), ctypes.byref(nh), ctypes.byref(it),
            ctypes.byref(err))
        L.check(st, "vdr_solve_gcr_record_device",
                allow=(L.OK, L.NOT_CONVERGED, L.BREAKDOWN))
        return nh.value, it.value, err.value, st

    @_device_call
    def solve_record_device(self, b, x, hist, tol=None, itmax=1000):
        """Jacobi-BiCGStab recording every iterate into hist (rows of N).
        Returns (recorded, iterations, relative residual, status)."""
        it, err, nh = ctypes.c_int(0), ctypes.c_double(0.0), ctypes.c_int(0)
        tol = self.problem.tol if tol is None else tol
        st = self.lib.vdr_solve_record_device(
            self.h, _ptr(b), _ptr(x), float(tol), int(itmax), _ptr(hist),
            int(hist.shape[0]), ctypes.byref(nh), ctypes.byref(it),
            ctypes.byref(err))
        L.check(st, "vdr_solve_record_device",
                allow=(L.OK, L.NOT_CONVERGED, L.BREAKDOWN))
        return nh.value, it.value, err.value, st

    @_device_call
    def solve_mixed_device(self, b, x, tol=None, inner_tol=1e-5, max_outer=20,
                           inner_itmax=1000):
        """FP64 refinement around FP32-operator inner solves.  Returns
        (outer corrections, inner iterations, FP64 relative residual,
        status)."""
        no, ni, err = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0.0)
        tol = self.problem.tol if tol is None else tol
        st = self.lib.vdr_solve_mixed_device(self.h, _ptr(b), _ptr(x),
                                             float(tol), float(inner_tol),
                                             int(max_outer), int(inner_itmax),
                                             ctypes.byref(no), ctypes.byref(ni),
                                             ctypes.byref(err))
        L.check(st, "vdr_solve_mixed_device",
                allow=(L.OK, L.NOT_CONVERGED, L.BREAKDOWN))
        return no.value, ni.value, err.value, st

    # ---- many right-hand sides: node-major N x K device arrays ----
    BLOCK_PRECISION = {"fp64": 0, "tf32": 1, "tf32x3": 2}

    def set_build_mode(self, mode="auto"):
        """How the element build gets the element geometry: "auto" (the
        mesh's geometric factors -- J^-1 and detJ at the Gauss points and
        the unit-diffusivity stiffness, 928 bytes per element -- formed on
        the GPU once and read by every later build) or "recompute" (the
        Jacobians evaluated from the coordinates at every build).  Marks
        the operator stale."""
        L.check(self.lib.vdr_set_build_mode(
            self.h, {"auto": 0, "recompute": 1}[mode]), "vdr_set_build_mode")

    def geometry_status(self):
        """(state, bytes): state 1 when the geometric factors are held (in
        `bytes` of device memory), 0 when not formed yet, -1 when the build
        cannot use them (no device memory, a factor outside the double-float
        window)."""
        st = ctypes.c_int(0)
        nb = ctypes.c_longlong(0)
        L.check(self.lib.vdr_geometry_status(self.h, ctypes.byref(st), ctypes.byref(nb)),
                "vdr_geometry_status")
        return st.value, nb.value

    def set_mixed_operator(self, mode="rounded"):
        """Inner operator of the mixed solve: "rounded" (the FP64 element
        matrices rounded to FP32), "recompute" (DR terms in FP32) or "half"
        (the Jacobi-scaled operator P A P D^-1 in binary16 with one
        power-of-two scale per element)."""
        L.check(self.lib.vdr_set_mixed_operator(
            self.h, {"rounded": 0, "recompute": 1, "half": 2}[mode]),
                "vdr_set_mixed_operator")

    @_device_call
    def apply_half_device(self, x, y):
        """y = A^ x with the binary16 inner operator A^ = P A P D^-1 (float32
        device vectors); needs set_mixed_operator("half")."""
        L.check(self.lib.vdr_apply_half_device(self.h, _ptr(x), _ptr(y)),
                "vdr_apply_half_device")

    def set_block_apply(self, variant="auto"):
        """Data movement of the tensor-core block apply: "auto" (default:
        the node tile, or for 64 columns the tcgen05 box apply when the
        first 64-column block solve measured it faster), "tcgen05" (64
        columns: 4 x 4 x 4-element box operators in tensor memory times the
        boxes' node rows on tcgen05), "tile" (node rows of 8 x 2 x 2-element
        boxes staged once in shared memory, mma.sync), all three on meshes
        in the canonical structured numbering ("lsu" otherwise), "lsu"
        (per-element row gathers and float4 atomics) or "bulk" (bulk copies
        and bulk reductions through shared memory)."""
        L.check(self.lib.vdr_set_block_apply(
            self.h, {"bulk": 0, "lsu": 1, "tile": 2, "tcgen05": 3, "auto": 4}[variant]),
            "vdr_set_block_apply")

    @_device_call
    def assemble_rhs_block_device(self, Q, B, cf=1.0):
        """B (N x K float64) = cf * f(Q_k) for the K x E per-element
        sources Q (caller's element order)."""
        K = int(Q.shape[0])
        L.check(self.lib.vdr_assemble_rhs_block_device(
            self.h, K, _ptr(Q), float(cf), _ptr(B)),
            "vdr_assemble_rhs_block_device")

    @_device_call
    def apply_block_device(self, X, Y, precision="fp64"):
        """Y = P A P X for the K columns of X (N x K; float64 for "fp64",
        float32 for "tf32" / "tf32x3")."""
        K = int(X.shape[1])
        L.check(self.lib.vdr_apply_block_device(
            self.h, K, _ptr(X), _ptr(Y), self.BLOCK_PRECISION[precision]),
            "vdr_apply_block_device")

    @_device_call
    def apply_block_accumulate_device(self, X, Y, precision="fp64"):
        """Y += P A P X (Y not zeroed first)."""
        K = int(X.shape[1])
        L.check(self.lib.vdr_apply_block_accumulate_device(
            self.h, K, _ptr(X), _ptr(Y), self.BLOCK_PRECISION[precision]),
            "vdr_apply_block_accumulate_device")

    @_device_call
    def solve_block_device(self, B, X, tol=None, inner_tol=1e-3,
                           precision="tf32x3", max_outer=30, inner_itmax=1000):
        """FP64 refinement around K simultaneous FP32 tensor-core inner
        solves.  Returns (outer corrections, inner iterations, per-column
        FP64 relative residuals, status)."""
        K = int(B.shape[1])
        no, ni = ctypes.c_int(0), ctypes.c_int(0)
        errs = np.zeros(K)
        tol = self.problem.tol if tol is None else tol
        st = self.lib.vdr_solve_block_device(
            self.h, K, self.BLOCK_PRECISION[precision], _ptr(B), _ptr(X),
            float(tol), float(inner_tol), int(max_outer), int(inner_itmax),
            ctypes.byref(no), ctypes.byref(ni), _dp(errs))
        L.check(st, "vdr_solve_block_device",
                allow=(L.OK, L.NOT_CONVERGED, L.BREAKDOWN))
        return no.value, ni.value, errs, st

    @_device_call
    def time_steps_device(self, t, nsteps, cf, rM, tol=None, itmax=1000):
        """The reference's time loop on the device (vdr_time_steps): t (device
        array) holds T_0 and returns T_nsteps.  Returns (masses, iterations,
        residuals, status, steps_done)."""
        masses = np.zeros(nsteps)
        iters = np.zeros(nsteps, dtype=np.int32)
        errs = np.zeros(nsteps)
        done = ctypes.c_int(0)
        tol = self.problem.tol if tol is None else tol
        st = self.lib.vdr_time_steps(self.h, int(nsteps), float(cf), float(rM),
                                     _ptr(t), float(tol), int(itmax),
                                     _dp(masses), _ip(iters), _dp(errs),
                                     ctypes.byref(done))
        L.check(st, "vdr_time_steps",
                allow=(L.OK, L.NOT_CONVERGED, L.BREAKDOWN))
        return masses, iters, errs, st, done.value

    @_device_call
    def true_residual_device(self, b, x):
        r = ctypes.c_double()
        L.check(self.lib.vdr_true_residual_device(self.h, _ptr(b), _ptr(x),
                                                  ctypes.byref(r)),
                "vdr_true_residual_device")
        return r.value

    @_device_call
    def mass_device(self, c):
        m = ctypes.c_double()
        L.check(self.lib.vdr_mass_device(self.h, _ptr(c), ctypes.byref(m)),
                "vdr_mass_device")
        return m.value

    def stats(self) -> dict:
        """Statistics of the most recent solve (vdr_last_solve_stats)."""
        st = L.VdrSolveStats()
        L.check(self.lib.vdr_last_solve_stats(self.h, ctypes.byref(st)),
                "vdr_last_solve_stats")
        return {k: getattr(st, k) for k in ("iterations", "status",
                                            "graph_launches",
                                            "kernel_launches", "breakdown")}

    def stream(self) -> int:
        return int(self.lib.vdr_stream(self.h) or 0)

    # -- lifetime ------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.vdr_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_FP = ctypes.POINTER(ctypes.c_float)


class LearnedNet:
    """The learned preconditioner bound to a Solver's mesh (libvdr's
    vdr_net_*): a 3-level 3D U-Net with BF16 weights, trained on the GPU by
    the library's own forward/backward kernels."""

    def __init__(self, solver: Solver, seed: int = 0):
        self.lib = solver.lib
        self.solver = solver
        h = ctypes.c_void_p()
        L.check(self.lib.vdr_net_create(solver.h, int(seed), ctypes.byref(h)),
                "vdr_net_create")
        self.h = h
        n = ctypes.c_longlong(0)
        L.check(self.lib.vdr_net_param_count(self.h, ctypes.byref(n)),
                "vdr_net_param_count")
        self.nparam = n.value

    CONV = {"mma": 0, "tcgen05": 1}

    def set_conv(self, mode: str):
        """Forward convolutions on "tcgen05" (fifth-generation tensor cores,
        TMA-staged operands, TMEM accumulators; the default where available)
        or "mma" (warp-level mma.sync)."""
        L.check(self.lib.vdr_net_set_conv(self.h, self.CONV[mode]), "vdr_net_set_conv")

    def conv_status(self):
        """(mode in use, status): status VDR_TIMEOUT (5) if a tcgen05
        convolution gave up waiting for its operands since the last call."""
        m = ctypes.c_int(-1)
        st = self.lib.vdr_net_conv_status(self.h, ctypes.byref(m))
        L.check(st, "vdr_net_conv_status", allow=(L.OK, L.TIMEOUT))
        return {0: "mma", 1: "tcgen05"}[m.value], st

    def get_params(self) -> np.ndarray:
        out = np.empty(self.nparam, dtype=np.float32)
        L.check(self.lib.vdr_net_get_params(self.h, out.ctypes.data_as(_FP)),
                "vdr_net_get_params")
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparam
        L.check(self.lib.vdr_net_set_params(self.h, p.ctypes.data_as(_FP)),
                "vdr_net_set_params")

    def get_grads(self) -> np.ndarray:
        out = np.empty(self.nparam, dtype=np.float32)
        L.check(self.lib.vdr_net_get_grads(self.h, out.ctypes.data_as(_FP)),
                "vdr_net_get_grads")
        return out

    @_device_call
    def update_features(self, feat_out=None) -> float:
        dbar = ctypes.c_double(0.0)
        L.check(self.lib.vdr_net_update_features(self.h, _ptr(feat_out),
                                                 ctypes.byref(dbar)),
                "vdr_net_update_features")
        return dbar.value

    @_device_call
    def set_features(self, feat, dbar: float):
        L.check(self.lib.vdr_net_set_features_device(self.h, _ptr(feat),
                                                     float(dbar)),
                "vdr_net_set_features_device")

    @_device_call
    def make_pair(self, b, xk, xstar, rhat, target):
        """Training pair from iterate xk of the solve A x = b (solution
        xstar): rhat = r/rms(r), target = (e - D^-1 r) dbar/rms(r)."""
        L.check(self.lib.vdr_net_make_pair_device(self.h, _ptr(b), _ptr(xk),
                                                  _ptr(xstar), _ptr(rhat),
                                                  _ptr(target)),
                "vdr_net_make_pair_device")

    @_device_call
    def forward(self, rhat, out):
        L.check(self.lib.vdr_net_forward_device(self.h, _ptr(rhat), _ptr(out)),
                "vdr_net_forward_device")

    @_device_call
    def loss_grad(self, rhat, target) -> float:
        loss = ctypes.c_double(0.0)
        L.check(self.lib.vdr_net_loss_grad_device(self.h, _ptr(rhat),
                                                  _ptr(target),
                                                  ctypes.byref(loss)),
                "vdr_net_loss_grad_device")
        return loss.value

    @_device_call
    def residual_loss_grad(self, rhat) -> float:
        """||rhat - A M(rhat)||^2 / ||rhat||^2 with the current operator, and
        the parameter gradients."""
        loss = ctypes.c_double(0.0)
        L.check(self.lib.vdr_net_residual_loss_grad_device(self.h, _ptr(rhat),
                                                           ctypes.byref(loss)),
                "vdr_net_residual_loss_grad_device")
        return loss.value

    @_device_call
    def train_step_residual(self, rhat, lr, want_loss=False):
        loss = ctypes.c_double(0.0)
        L.check(self.lib.vdr_net_train_step_residual_device(
            self.h, _ptr(rhat), float(lr),
            ctypes.byref(loss) if want_loss else None),
            "vdr_net_train_step_residual_device")
        return loss.value if want_loss else None

    @_device_call
    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8):
        L.check(self.lib.vdr_net_adam_step(self.h, float(lr), float(beta1),
                                           float(beta2), float(eps)),
                "vdr_net_adam_step")

    @_device_call
    def train_step(self, rhat, target, lr, want_loss=False):
        loss = ctypes.c_double(0.0)
        L.check(self.lib.vdr_net_train_step_device(
            self.h, _ptr(rhat), _ptr(target), float(lr),
            ctypes.byref(loss) if want_loss else None),
            "vdr_net_train_step_device")
        return loss.value if want_loss else None

    def set_smoothing(self, steps=1, omega=1.0):
        """Jacobi post-smoothing steps after the network (0 = none)."""
        L.check(self.lib.vdr_net_set_smoothing(self.h, int(steps), float(omega)),
                "vdr_net_set_smoothing")

    @_device_call
    def precondition(self, x, y):
        L.check(self.lib.vdr_net_precondition_device(self.h, _ptr(x), _ptr(y)),
                "vdr_net_precondition_device")

    def close(self):
        if getattr(self, "h", None):
            self.lib.vdr_net_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kernel_launch_count() -> int:
    """Kernels libvdr.so has launched in this process (vdr_kernel_launch_count)."""
    return int(L.load_library().vdr_kernel_launch_count())


def kernel_dbcg_simple(N, B, X, TOL, ITMAX, BB, ISS, DIAG, NAX, NAY, NAZ,
                       bc_dirichlet):
    """The reference's solve call.  Returns (X, ITER, ERR); X is a new array
    holding the solution (the C symbol itself writes X in place)."""
    lib = L.load_library()
    n = ctypes.c_int(int(N))
    b = _f64(B)
    x = np.array(X, dtype=np.float64, copy=True)
    tol = ctypes.c_double(float(TOL))
    itmax = ctypes.c_int(int(ITMAX))
    it = ctypes.c_int(0)
    err = ctypes.c_double(0.0)
    bb, iss, dg = _f64(BB), _i32(ISS), _f64(DIAG)
    nax, nay, naz = (ctypes.c_int(int(v)) for v in (NAX, NAY, NAZ))
    bc = _i32(bc_dirichlet)
    lib.kernel_dbcg_simple_(ctypes.byref(n), _dp(b), _dp(x), ctypes.byref(tol),
                            ctypes.byref(itmax), ctypes.byref(it),
                            ctypes.byref(err), _dp(bb), _ip(iss), _dp(dg),
                            ctypes.byref(nax), ctypes.byref(nay),
                            ctypes.byref(naz), _ip(bc))
    return x, it.value, err.value


def _host_f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(ctypes.c_void_p)


def format_result_txt(xx, yy, zz, t, scale=1e6, out=None):
    """The text of the reference's T_sssss.TXT for node arrays xx, yy, zz
    and the field t: per node x, y, z, t * scale in Fortran format
    (e12.5, 2x, e12.5, 2x, e12.5, 2x, e12.5), 55 bytes per line.  Returns
    bytes, or fills and returns `out` (a uint8 array of 55 * N bytes)."""
    lib = L.load_library()
    arrs = [_host_f64(a) for a in (xx, yy, zz, t)]
    n = arrs[0][0].size
    buf = out if out is not None else np.empty(55 * n, dtype=np.uint8)
    if buf.dtype != np.uint8 or buf.size != 55 * n or not buf.flags.c_contiguous:
        raise ValueError("out must be a contiguous uint8 array of 55 * N bytes")
    L.check(lib.vdr_format_result_txt(buf.ctypes.data_as(ctypes.c_void_p), n,
                                      *(p for _, p in arrs), float(scale)),
            "vdr_format_result_txt")
    return buf if out is not None else buf.tobytes()


def write_result_txt(directory, step, xx, yy, zz, t, scale=1e6):
    """Writes directory/T_sssss.TXT as the reference's time step does."""
    lib = L.load_library()
    arrs = [_host_f64(a) for a in (xx, yy, zz, t)]
    L.check(lib.vdr_write_result_txt(str(directory).encode(), int(step),
                                     arrs[0][0].size, *(p for _, p in arrs),
                                     float(scale)), "vdr_write_result_txt")


def write_slices_txt(directory, step, nax, nay, naz, xx, yy, zz, t, scale=1e6):
    """Writes the X_/Y_/Z_sssss_iii.TXT slice files that the reference's
    vanadis_files splits from T_sssss.TXT (node grid nax x nay x naz)."""
    lib = L.load_library()
    arrs = [_host_f64(a) for a in (xx, yy, zz, t)]
    L.check(lib.vdr_write_slices_txt(str(directory).encode(), int(step), int(nax),
                                     int(nay), int(naz), *(p for _, p in arrs),
                                     float(scale)), "vdr_write_slices_txt")
