"""The C-ABI library: builds for sm_103a, loads, and exports every symbol
include/vdr.h declares (no GPU calls here)."""
import ctypes
import os
import re
import subprocess

from helpers import HERE

ROOT = os.path.dirname(HERE)


def declared_functions():
    src = open(os.path.join(ROOT, "include", "vdr.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b([a-z_][a-z0-9_]*)\s*\(", src)) -
                  {"if", "sizeof"})


def test_header_lists_reference_entry_point():
    assert "kernel_dbcg_simple_" in declared_functions()


def test_library_exports_every_declared_symbol(vdr):
    path = vdr.build_library()
    out = subprocess.run(["nm", "-D", "--defined-only", path],
                         capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing


def test_python_binding_covers_header(vdr):
    from importlib import import_module
    lib_mod = import_module(vdr.__name__ + "._lib")
    assert set(declared_functions()) == set(lib_mod.SIGNATURES)


def test_library_loads_without_gpu(vdr):
    lib = vdr.load_library()
    assert lib.vdr_last_error() is not None
    o = import_opts(vdr)
    assert lib.vdr_default_options(ctypes.byref(o)) == 0
    assert o.dr_variant == 2 and o.iters_per_graph == 8


def import_opts(vdr):
    from importlib import import_module
    return import_module(vdr.__name__ + "._lib").VdrOptions()
