"""The ISO_C_BINDING module (fortran/vdr_iso_c.f90) against the C ABI
(include/vdr.h), read as text (no Fortran compiler is needed):

* every bind(c) interface names a function the header declares, with the
  same result (integer(c_int) function <-> int, subroutine <-> void) and,
  argument by argument, the C type its Fortran declaration passes: VALUE
  scalars by value, everything else by address (arrays, intent(out)
  scalars, derived types);
* the vdr_options derived type has the C struct's fields in order;
* the status-code parameters equal the header's #defines.
"""
import os
import re

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
F90 = os.path.join(ROOT, "vanadis_solver-directional_residual_gb300", "fortran",
                   "vdr_iso_c.f90")
HDR = os.path.join(ROOT, "include", "vdr.h")


def fortran_lines():
    """Source lines with comments stripped and & continuations joined."""
    out, cur = [], ""
    for raw in open(F90):
        line = raw.split("!", 1)[0].rstrip()
        if not line.strip():
            continue
        if cur:
            line = line.lstrip()
            if line.startswith("&"):
                line = line[1:]
        if line.endswith("&"):
            cur += line[:-1] + " "
            continue
        out.append(cur + line)
        cur = ""
    return out


def fortran_interfaces():
    lines = fortran_lines()
    items, i = {}, 0
    head = re.compile(r"\s*(integer\(c_int\)\s+function|subroutine)\s+(\w+)\s*"
                      r"\(([^)]*)\)\s*bind\(c,\s*name=\"(\w+)\"\)", re.I)
    while i < len(lines):
        m = head.match(lines[i])
        if not m:
            i += 1
            continue
        kind = "int" if "function" in m.group(1).lower() else "void"
        args = [a.strip().lower() for a in m.group(3).split(",") if a.strip()]
        decl = {}
        i += 1
        while not re.match(r"\s*end\s+(function|subroutine)", lines[i], re.I):
            d = re.match(r"\s*(type\(\w+\)|real\(\w+\)|integer\(\w+\)|"
                         r"character\(kind=\w+\))([^:]*)::(.*)", lines[i], re.I)
            if d:
                base = re.search(r"\((?:kind=)?(\w+)\)", d.group(1)).group(1).lower()
                value = "value" in d.group(2).lower()
                for v in re.split(r",(?![^(]*\))", d.group(3)):
                    v = v.strip().lower()
                    name = v.split("(")[0].strip()
                    decl[name] = (base, value, "(" in v)
            i += 1
        items[m.group(4)] = (kind, [(a, decl[a]) for a in args])
        i += 1
    return items


def c_prototypes():
    text = open(HDR).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    protos = {}
    for m in re.finditer(r"\b(int|void|long long|const char \*)\s*(\w+)\s*\(([^;{]*?)\)\s*;",
                         text):
        args = []
        body = m.group(3).strip()
        if body and body != "void":
            for a in body.split(","):
                a = a.replace("const", " ").strip()
                depth = a.count("*")
                base = a.replace("*", " ").split()[0]
                args.append((base, depth))
        protos[m.group(2)] = (m.group(1), args)
    return protos


def expected_c(base, value):
    """The C (type, pointer depth) a Fortran dummy argument passes."""
    if base == "c_ptr":
        return ("vdr_handle", 1 if value else 2)
    # (the header parser keeps the first word of a type: "long long" -> "long")
    c = {"c_double": "double", "c_int": "int", "c_long": "long",
         "c_long_long": "long", "c_char": "char",
         "vdr_options": "vdr_options"}[base]
    return (c, 0 if value else 1)


INTERFACES = fortran_interfaces()


def test_module_declares_interfaces():
    assert len(INTERFACES) >= 15
    assert "kernel_dbcg_simple_" in INTERFACES


@pytest.mark.parametrize("bind_name", sorted(INTERFACES))
def test_interface_matches_c_prototype(bind_name):
    protos = c_prototypes()
    assert bind_name in protos, bind_name
    kind, fargs = INTERFACES[bind_name]
    ckind, cargs = protos[bind_name]
    assert kind == ckind, (kind, ckind)
    assert len(fargs) == len(cargs), (fargs, cargs)
    for (name, (base, value, array)), (cbase, cdepth) in zip(fargs, cargs):
        want = expected_c(base, value)
        assert (cbase, cdepth) == want, (bind_name, name, (cbase, cdepth), want)
        assert not (value and array), (bind_name, name)


def test_options_type_matches_c_struct():
    src = "\n".join(fortran_lines())
    body = re.search(r"type, bind\(c\) :: vdr_options(.*?)end type", src, re.S).group(1)
    fnames = []
    for d in re.findall(r"::(.*)", body):
        fnames += [v.strip().split("(")[0] for v in d.split(",") if v.strip()]
    text = re.sub(r"/\*.*?\*/", " ", open(HDR).read(), flags=re.S)
    cbody = re.search(r"typedef struct vdr_options \{(.*?)\} vdr_options;", text, re.S).group(1)
    cnames = [re.sub(r"\[.*\]", "", d.split()[-1]) for d in cbody.split(";") if d.strip()]
    assert fnames == cnames


def test_status_codes_match_header():
    src = "\n".join(fortran_lines())
    hdr = open(HDR).read()
    for name, val in re.findall(r"(VDR_\w+)\s*=\s*(\d+)", src):
        m = re.search(r"#define\s+%s\s+(\d+)" % name, hdr)
        assert m and int(m.group(1)) == int(val), name
