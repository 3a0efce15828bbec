"""The reference's text outputs of a time step (host side, no GPU):

* the oracle's Fortran Ew.d edit against known answers of the E12.5 rule;
* the library's T_sssss.TXT text against the oracle's restatement of
  vanadis_full_DR_OpenMP_timing.for:797-806, byte for byte, over values of
  every magnitude, sign, zero, exact ties, NaN and infinities;
* the library's X/Y/Z slice files against the oracle's restatement of
  vanadis_files (:1089-1184), which reads the written T file back and
  splits it, byte for byte;
* argument and I/O errors.
"""
import os

import numpy as np
import pytest

# Ew.d with w = 12, d = 5: sign or blank, "0.", 5 significant digits, then
# E+ee, or +eee when the exponent needs three digits.
KNOWN = [
    (1.0, " 0.10000E+01"),
    (0.0, " 0.00000E+00"),
    (-123.456, "-0.12346E+03"),
    (9.999996, " 0.10000E+02"),
    (-0.00012345678, "-0.12346E-03"),
    (6.02e23, " 0.60200E+24"),
    (1e-150, " 0.10000-149"),
    (5e-100, " 0.50000E-99"),
    (5e-101, " 0.50000-100"),
    (1.7976931348623157e308, " 0.17977+309"),
    (5e-324, " 0.49407-323"),
    (1.23455, " 0.12346E+01"),   # the double is 1.23455000000000003624...
    (1.03125, " 0.10312E+01"),   # an exact binary tie: to the even digit
    (99999.5, " 0.10000E+06"),   # an exact tie rounding up to the even 10000
    (float("nan"), "         NaN"),
    (float("inf"), "    Infinity"),
    (float("-inf"), "   -Infinity"),
]


@pytest.mark.parametrize("v,text", KNOWN)
def test_oracle_fortran_e12_5_known_answers(v, text):
    from oracle.textio import fortran_e
    assert fortran_e(v) == text


def edge_values():
    rng = np.random.default_rng(11)
    v = np.concatenate([
        rng.standard_normal(400) * 10.0 ** rng.integers(-310, 309, 400),
        rng.uniform(-1, 1, 200),
        [0.0, -0.0, 1.03125, 99999.5, 0.5, 2.5e-5, 1e-100, 9.99995e99,
         np.nextafter(1.0, 2.0), float("nan"), float("inf"), float("-inf"),
         5e-324, 1e308],
    ])
    with np.errstate(over="ignore"):
        return v.astype(np.float64)


def test_library_result_text_matches_oracle(vdr):
    from oracle.textio import result_txt
    v = edge_values()
    n = v.size
    rng = np.random.default_rng(3)
    xx, yy, zz = (rng.uniform(-5e3, 5e3, n) for _ in range(3))
    for scale in (1e6, 1.0):
        got = vdr.format_result_txt(xx, yy, zz, v, scale)
        with np.errstate(over="ignore", invalid="ignore"):
            want = result_txt(xx, yy, zz, v, scale)
        assert len(got) == 55 * n
        assert got == want


def test_library_files_match_oracle_split(vdr, tmp_path):
    """T_00007.TXT and its slices on a 6 x 4 x 3 node grid: the library's
    files equal the oracle's T text and vanadis_files' split of it."""
    from oracle.textio import result_txt, split_result_txt
    m = vdr.problems.structured_mesh(5, 3, 2, jitter=0.1, seed=4)
    n = m.nnode
    t = np.random.default_rng(8).standard_normal(n) * 1e-7
    t[3] = 0.0
    step = 7
    vdr.write_result_txt(tmp_path, step, m.xx, m.yy, m.zz, t)
    vdr.write_slices_txt(tmp_path, step, m.nax, m.nay, m.naz, m.xx, m.yy, m.zz, t)
    text = result_txt(m.xx, m.yy, m.zz, t, 1e6)
    assert (tmp_path / "T_00007.TXT").read_bytes() == text
    want = split_result_txt(text, m.nax, m.nay, m.naz, step)
    names = sorted(p for p in os.listdir(tmp_path) if p != "T_00007.TXT")
    assert names == sorted(want)
    for name, body in want.items():
        assert (tmp_path / name).read_bytes() == body, name


def test_large_grid_threads_match_oracle(vdr):
    """Enough lines for the multi-threaded path."""
    from oracle.textio import result_txt
    n = 70001
    rng = np.random.default_rng(21)
    xx, yy, zz, t = (rng.standard_normal(n) * 10.0 ** rng.integers(-30, 30, n)
                     for _ in range(4))
    assert vdr.format_result_txt(xx, yy, zz, t, 1e6) == result_txt(xx, yy, zz, t, 1e6)


def test_text_output_errors(vdr, tmp_path):
    import importlib
    L = importlib.import_module(vdr.__name__ + "._lib")
    x = np.zeros(8)
    with pytest.raises(L.VdrError) as e:
        vdr.write_slices_txt(tmp_path, 1, 1000, 1, 1, *(np.zeros(1000),) * 4)
    assert e.value.status == L.BAD_ARGUMENT
    with pytest.raises(L.VdrError) as e:
        vdr.write_result_txt(tmp_path, 100000, x, x, x, x)
    assert e.value.status == L.BAD_ARGUMENT
    with pytest.raises(L.VdrError) as e:
        vdr.write_result_txt(tmp_path / "missing" / "dir", 1, x, x, x, x)
    assert e.value.status == L.IO_ERROR
