"""GB300 (sm_103a) element-by-element HEX8 directional-residual solve.

A drop-in for the solve path of the Vanadis transport model: the reference
driver's ``kernel_dbcg_simple_`` entry point, plus a handle API that keeps
mesh, fields and operator resident on the GPU and recomputes the DR element
terms there.  The compute lives in ``lib/libvdr.so`` (hand-written CUDA for
sm_103a + C++ host runtime, C ABI in ``include/vdr.h``); this package is its
Python host binding.
"""
from . import learned, problems
from ._lib import (VdrError, build_library, last_error, library_path,
                   load_library)
from .solver import (LearnedNet, Options, Solver, format_result_txt,
                     kernel_dbcg_simple, kernel_launch_count, write_result_txt,
                     write_slices_txt)

__all__ = ["problems", "learned", "Options", "Solver", "LearnedNet", "kernel_dbcg_simple",
           "kernel_launch_count", "VdrError", "format_result_txt",
           "write_result_txt", "write_slices_txt",
           "build_library", "load_library", "library_path", "last_error"]
