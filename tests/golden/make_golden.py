"""Regenerates the golden fixtures in this folder from the reference tree.

Run where the reference is mounted (default /root/reference, or
$VDR_REFERENCE_ROOT) after `bash oracle/build_ref.sh`:

    python tests/golden/make_golden.py

Writes
  vanadis_log_kat.json  the reference's only recorded run: mesh axis
                        coordinates (wsp_na_o, vanadis_full_DR_OpenMP_timing.for
                        :91-139), configuration (src_v2026_2_1/vanadis.cfg:5),
                        and the printed dominance factor, BiCG iteration
                        counts, residuals and masses (vanadis_log.txt:42-240)
  ref_colors.npz        element colours and per-colour lists computed by the
                        reference's own generate_hex8_colors /
                        build_color_element_lists
                        (cudatest_coloring_gtx1060_optimized.cu:50-106),
                        compiled from its sources into oracle/_ref
"""
from __future__ import annotations

import ctypes
import json
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("VDR_REFERENCE_ROOT", "/root/reference")

# (nax, nay, naz) node counts whose colourings are recorded.
COLOR_MESHES = [(2, 2, 2), (3, 2, 2), (4, 5, 3), (7, 20, 20), (33, 33, 17),
                (6, 3, 9)]


def parse_axes():
    src = open(os.path.join(REF, "src_updates",
                            "vanadis_full_DR_OpenMP_timing.for"),
               encoding="latin-1").read()
    axes = {}
    for ax in ("dx", "dy", "dz"):
        vals = {}
        for m in re.finditer(r"^\s*%s\((\d+)\)\s*=\s*([-+0-9.]+)d\+?0*([-+]?\d*)"
                             % ax, src, re.M):
            vals[int(m.group(1))] = float(m.group(2)) * 10.0 ** int(m.group(3) or 0)
        axes[ax] = [vals[k] for k in sorted(vals)]
    return axes


def parse_cfg():
    lines = open(os.path.join(REF, "src_v2026_2_1", "vanadis.cfg"),
                 encoding="latin-1").read().splitlines()
    nums = [float(t.replace("D", "E")) for t in lines[5].split()]
    keys = ["Q", "K", "P", "V1", "V2", "V3", "ALPHA"]
    return dict(zip(keys, nums))


def parse_log():
    txt = open(os.path.join(REF, "src_v2026_2_1", "vanadis_log.txt"),
               encoding="latin-1").read()
    dom = [float(v) for v in re.findall(r"wspolczynnik dominacji\s+(\S+)", txt)]
    its = [int(v) for v in re.findall(r"number of iterations:\s+(\d+)", txt)]
    res = [float(v.replace("E", "e")) for v in
           re.findall(r"residual norm:\s+(\S+)", txt)]
    mass = [float(v) for v in re.findall(r"masa=\s+(\S+)", txt)]
    times = [int(v) for v in re.findall(r"czas=\s+(\d+)", txt)]
    dd = re.findall(r"Diagonally dominant matrix \[T/F\]\s+(\S)", txt)
    return dict(dominance_factor=dom[0], dominance_all_steps=dom,
                diagonally_dominant=(dd[0] == "T"), iterations=its,
                residuals=res, masses=mass, times=times)


def ref_colors():
    so = os.path.join(ROOT, "oracle", "_ref", "libref_coloring.so")
    L = ctypes.CDLL(so)
    gen = getattr(L, "_Z20generate_hex8_colorsiiiPi")
    lists = getattr(L, "_Z25build_color_element_listsiPKiPiS1_S1_")
    IP = ctypes.POINTER(ctypes.c_int)
    gen.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, IP]
    lists.argtypes = [ctypes.c_int, IP, IP, IP, IP]
    out = {}
    for nax, nay, naz in COLOR_MESHES:
        E = (nax - 1) * (nay - 1) * (naz - 1)
        col = np.zeros(E, dtype=np.int32)
        gen(nax, nay, naz, col.ctypes.data_as(IP))
        elems = np.zeros(E, dtype=np.int32)
        offs = np.zeros(9, dtype=np.int32)
        counts = np.zeros(8, dtype=np.int32)
        lists(E, col.ctypes.data_as(IP), elems.ctypes.data_as(IP),
              offs.ctypes.data_as(IP), counts.ctypes.data_as(IP))
        key = "%d_%d_%d" % (nax, nay, naz)
        out["colors_" + key] = col
        out["elems_" + key] = elems
        out["offsets_" + key] = offs
        out["counts_" + key] = counts
    return out


def main():
    kat = dict(source="src_v2026_2_1/vanadis_log.txt (VANADIS.FOR v1.08 + "
                      "cudatest.cu), mesh from vanadis_full_DR_OpenMP_timing."
                      "for:91-139, cfg from src_v2026_2_1/vanadis.cfg:5",
               nax=7, nay=20, naz=20, dt=100, steps=20, tol=1e-8, itmax=1000,
               source_element_1based=1083, dr_variant="VF", mask="VF")
    kat.update(parse_axes())
    kat["cfg"] = parse_cfg()
    kat["log"] = parse_log()
    with open(os.path.join(HERE, "vanadis_log_kat.json"), "w") as f:
        json.dump(kat, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "ref_colors.npz"), **ref_colors())
    print("wrote vanadis_log_kat.json and ref_colors.npz")


if __name__ == "__main__":
    main()
