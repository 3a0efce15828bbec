"""ctypes binding of libvdr.so (the C ABI declared in include/vdr.h).

The library is the only compute path: if it is missing or cannot load, the
package raises instead of falling back to anything else."""
from __future__ import annotations

import ctypes
import os

from . import build as _build

_lib = None

OK, NOT_CONVERGED, BREAKDOWN, CUDA_ERROR, BAD_ARGUMENT, TIMEOUT, IO_ERROR = range(7)
STATUS_NAMES = {0: "ok", 1: "not converged", 2: "breakdown",
                3: "cuda error", 4: "bad argument", 5: "timeout",
                6: "i/o error"}

DR_OT, DR_GP, DR_VF = 0, 1, 2
SCATTER_AUTO, SCATTER_ATOMIC, SCATTER_COLOR, SCATTER_WARP = 0, 1, 2, 3
APPLY_AUTO, APPLY_STORED, APPLY_MATRIX_FREE = 0, 1, 2
SOLVER_BICGSTAB, SOLVER_BICG = 0, 1
STORE_AUTO, STORE_FP64, STORE_DF = 0, 1, 2
PRECISION_FP64, PRECISION_MIXED = 0, 1


class VdrOptions(ctypes.Structure):
    _fields_ = [("dr_variant", ctypes.c_int), ("scatter", ctypes.c_int),
                ("apply_mode", ctypes.c_int), ("solver", ctypes.c_int),
                ("iters_per_graph", ctypes.c_int), ("device", ctypes.c_int),
                ("matrix_storage", ctypes.c_int), ("precision", ctypes.c_int),
                ("reserved", ctypes.c_int * 8)]


class VdrApplyTuning(ctypes.Structure):
    _fields_ = [("apply_blocks_per_sm", ctypes.c_int),
                ("half_blocks_per_sm", ctypes.c_int),
                ("block_tile_y", ctypes.c_int), ("block_halves", ctypes.c_int),
                ("grid_candidates", ctypes.c_int * 5),
                ("apply_ms", ctypes.c_float * 5), ("half_ms", ctypes.c_float * 5),
                ("block_ms", ctypes.c_float * 4), ("block_tcgen05", ctypes.c_int)]


class VdrSolveStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int), ("status", ctypes.c_int),
                ("graph_launches", ctypes.c_int),
                ("kernel_launches", ctypes.c_int), ("breakdown", ctypes.c_int),
                ("reserved", ctypes.c_int * 3)]


# Every symbol include/vdr.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_i = ctypes.c_int
_d = ctypes.c_double
_f = ctypes.c_float
_F = ctypes.POINTER(ctypes.c_float)
SIGNATURES = {
    "vdr_default_options": (_i, [ctypes.POINTER(VdrOptions)]),
    "vdr_create": (_i, [ctypes.POINTER(_P), _i, _i, _D, _D, _D, _I, _I,
                        ctypes.POINTER(VdrOptions)]),
    "vdr_set_fields": (_i, [_P, _D, _D, _D, _D, _d]),
    "vdr_set_dirichlet": (_i, [_P, _I]),
    "vdr_set_operator": (_i, [_P, _d, _d]),
    "vdr_apply": (_i, [_P, _D, _D, _i]),
    "vdr_apply_device": (_i, [_P, _P, _P, _i]),
    "vdr_apply_accumulate_device": (_i, [_P, _P, _P, _i]),
    "vdr_apply32_device": (_i, [_P, _P, _P, _i]),
    "vdr_assemble_rhs": (_i, [_P, _d, _d, _D, _D]),
    "vdr_assemble_rhs_device": (_i, [_P, _d, _d, _P, _P]),
    "vdr_get_diag": (_i, [_P, _D]),
    "vdr_get_element_matrices": (_i, [_P, _D]),
    "vdr_get_element_matrices_device": (_i, [_P, _P]),
    "vdr_solve": (_i, [_P, _D, _D, _d, _i, _I, _D]),
    "vdr_solve_device": (_i, [_P, _P, _P, _d, _i, _I, _D]),
    "vdr_solve_mixed_device": (_i, [_P, _P, _P, _d, _d, _i, _i, _I, _I, _D]),
    "vdr_assemble_rhs_block_device": (_i, [_P, _i, _P, _d, _P]),
    "vdr_set_block_apply": (_i, [_P, _i]),
    "vdr_diag_wait_timeout": (_i, [_P]),
    "vdr_diag_barrier_timeout": (_i, [_P]),
    "vdr_set_mixed_operator": (_i, [_P, _i]),
    "vdr_set_build_mode": (_i, [_P, _i]),
    "vdr_diag_beta_vf": (_i, [_i, _D, _D]),
    "vdr_geometry_status": (_i, [_P, _I, ctypes.POINTER(ctypes.c_longlong)]),
    "vdr_apply_half_device": (_i, [_P, _P, _P]),
    "vdr_apply_block_device": (_i, [_P, _i, _P, _P, _i]),
    "vdr_apply_block_accumulate_device": (_i, [_P, _i, _P, _P, _i]),
    "vdr_solve_block_device": (_i, [_P, _i, _i, _P, _P, _d, _d, _i, _i, _I,
                                    _I, _D]),
    "vdr_true_residual_device": (_i, [_P, _P, _P, _D]),
    "vdr_set_segments": (_i, [_P, _i, _I]),
    "vdr_solve_segmented_device": (_i, [_P, _P, _P, _d, _i, _I, _D, _I]),
    "vdr_segment_tuning": (_i, [_P, _I, _I]),
    "vdr_apply_tuning": (_i, [_P, ctypes.POINTER(VdrApplyTuning)]),
    "vdr_net_create": (_i, [_P, ctypes.c_ulonglong, ctypes.POINTER(_P)]),
    "vdr_net_destroy": (_i, [_P]),
    "vdr_net_param_count": (_i, [_P, ctypes.POINTER(ctypes.c_longlong)]),
    "vdr_net_get_params": (_i, [_P, _F]),
    "vdr_net_set_params": (_i, [_P, _F]),
    "vdr_net_get_grads": (_i, [_P, _F]),
    "vdr_net_update_features": (_i, [_P, _P, _D]),
    "vdr_net_set_features_device": (_i, [_P, _P, _d]),
    "vdr_net_make_pair_device": (_i, [_P, _P, _P, _P, _P, _P]),
    "vdr_net_forward_device": (_i, [_P, _P, _P]),
    "vdr_net_loss_grad_device": (_i, [_P, _P, _P, _D]),
    "vdr_net_adam_step": (_i, [_P, _f, _f, _f, _f]),
    "vdr_net_residual_loss_grad_device": (_i, [_P, _P, _D]),
    "vdr_net_train_step_residual_device": (_i, [_P, _P, _f, _D]),
    "vdr_net_train_step_device": (_i, [_P, _P, _P, _f, _D]),
    "vdr_net_precondition_device": (_i, [_P, _P, _P]),
    "vdr_net_set_smoothing": (_i, [_P, _i, _d]),
    "vdr_net_set_conv": (_i, [_P, _i]),
    "vdr_net_conv_status": (_i, [_P, _I]),
    "vdr_solve_learned_device": (_i, [_P, _P, _P, _P, _d, _i, _i, _I, _D, _I]),
    "vdr_solve_gcr_device": (_i, [_P, _P, _P, _P, _d, _i, _i, _i, _I, _D,
                                  _I]),
    "vdr_solve_learned_hybrid_device": (_i, [_P, _P, _P, _P, _d, _i, _i, _I,
                                             _D]),
    "vdr_solve_gcr_record_device": (_i, [_P, _P, _P, _P, _d, _i, _i, _P, _i,
                                         _I, _I, _D]),
    "vdr_solve_record_device": (_i, [_P, _P, _P, _d, _i, _P, _i, _I, _I, _D]),
    "vdr_time_steps": (_i, [_P, _i, _d, _d, _P, _d, _i, _D, _I, _D, _I]),
    "vdr_mass": (_i, [_P, _D, _D]),
    "vdr_mass_device": (_i, [_P, _P, _D]),
    "vdr_color_elements": (_i, [_i, _i, _I, _I]),
    "vdr_last_solve_stats": (_i, [_P, ctypes.POINTER(VdrSolveStats)]),
    "vdr_kernel_launch_count": (ctypes.c_longlong, []),
    "vdr_stream": (_P, [_P]),
    "vdr_destroy": (_i, [_P]),
    "vdr_last_error": (ctypes.c_char_p, []),
    "vdr_write_result_txt": (_i, [ctypes.c_char_p, _i, ctypes.c_long, _P, _P,
                                  _P, _P, _d]),
    "vdr_format_result_txt": (_i, [_P, ctypes.c_long, _P, _P, _P, _P, _d]),
    "vdr_write_slices_txt": (_i, [ctypes.c_char_p, _i, _i, _i, _i, _P, _P, _P,
                                  _P, _d]),
    "kernel_dbcg_simple_": (None, [_I, _D, _D, _D, _I, _I, _D, _D, _I, _D,
                                   _I, _I, _I, _I]),
    "vdr_bicg_noalloc_device": (_i, [_i, _i, _i, _i, _P, _P, _d, _i, _P, _P,
                                     _P, _P, _P, _I, _D]),
}


def library_path() -> str:
    return _build.LIB_PATH


def build_library(force: bool = False) -> str:
    return _build.build(force=force)


def load_library():
    """Load libvdr.so (it must have been built; raises otherwise)."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(
            "libvdr.so not built (%s); run __graft_entry__.build()" % path)
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    return load_library().vdr_last_error().decode(errors="replace")


class VdrError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        super().__init__("%s: %s (%s)" % (where, STATUS_NAMES.get(status, status),
                                          last_error()))


def check(status: int, where: str, allow=(OK,)) -> int:
    if status not in allow:
        raise VdrError(status, where)
    return status
