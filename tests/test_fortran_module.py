"""include/funwave_gpu.F90 against include/funwave_gpu.h, without a Fortran
compiler: the BIND(C) type FW_PARAMS has the fields of fw_params in the same
order with the matching kinds (so a Fortran caller's object has the C
layout), every interface binds a function the header declares and the
library exports, with the same number of arguments, every header function
has an interface, and the status constants agree.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "include", "funwave_gpu.F90")
HDR = os.path.join(ROOT, "include", "funwave_gpu.h")

KIND = {"int": "INTEGER(C_INT)", "double": "REAL(C_DOUBLE)"}


def _fortran_lines():
    """Free-form source with comments removed and & continuations joined."""
    out, cur = [], ""
    for raw in open(F90).read().splitlines():
        line = raw.split("!", 1)[0].rstrip()
        if not line.strip():
            continue
        if cur:
            line = line.lstrip()
            if line.startswith("&"):
                line = line[1:]
        if line.endswith("&"):
            cur += line[:-1]
            continue
        out.append(cur + line)
        cur = ""
    return out


def _c_source():
    s = open(HDR).read()
    s = re.sub(r"/\*.*?\*/", " ", s, flags=re.S)
    return s


def _c_params_fields():
    s = _c_source()
    body = re.search(r"typedef struct fw_params\s*\{(.*?)\}\s*fw_params;", s, re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        typ, names = decl.split(None, 1)
        fields += [(n.strip().lower(), KIND[typ]) for n in names.split(",")]
    return fields


def _f_params_fields():
    lines = _fortran_lines()
    i = next(k for k, l in enumerate(lines) if re.match(r"\s*TYPE\s*,\s*BIND\(C\)\s*::\s*FW_PARAMS", l, re.I))
    fields = []
    for l in lines[i + 1:]:
        if re.match(r"\s*END\s+TYPE", l, re.I):
            break
        typ, names = l.split("::")
        fields += [(n.strip().lower(), typ.strip().upper()) for n in names.split(",")]
    return fields


def _c_functions():
    """{name: number of parameters} of the header's prototypes."""
    s = _c_source()
    out = {}
    for m in re.finditer(r"^\s*(?:int|void|const char|long long)\s*\*?\s*(fw_\w+)\s*\(([^;]*?)\)\s*;", s, re.M | re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else len(args.split(","))
    return out


def _f_interfaces():
    """[(fortran name, bound C name, dummy names, declared names)]."""
    lines = _fortran_lines()
    out = []
    head = re.compile(r"\s*(?:[\w(),]+\s+)?(?:FUNCTION|SUBROUTINE)\s+(\w+)\s*\(([^)]*)\)\s*BIND\(C,\s*NAME=\"(\w+)\"\)",
                      re.I)
    k = 0
    while k < len(lines):
        m = head.match(lines[k])
        if not m:
            k += 1
            continue
        dummies = [a.strip().lower() for a in m.group(2).split(",") if a.strip()]
        declared = set()
        k += 1
        while not re.match(r"\s*END\s+(FUNCTION|SUBROUTINE)", lines[k], re.I):
            if "::" in lines[k] and not re.match(r"\s*IMPORT", lines[k], re.I):
                for n in lines[k].split("::")[1].split(","):
                    declared.add(re.sub(r"\(.*", "", n).strip().lower())
            k += 1
        out.append((m.group(1), m.group(3), dummies, declared))
    return out


def test_fw_params_type_matches_header():
    c, f = _c_params_fields(), _f_params_fields()
    assert [n for n, _ in f] == [n for n, _ in c], "field names or order differ"
    for (n, kc), (_, kf) in zip(c, f):
        assert kc == kf, "%s: C %s, Fortran %s" % (n, kc, kf)
    assert ("track_roller", "INTEGER(C_INT)") in f and ("track_radiation", "INTEGER(C_INT)") in f


def test_every_interface_binds_a_declared_function_with_its_arity():
    cf = _c_functions()
    seen = set()
    for fname, cname, dummies, declared in _f_interfaces():
        assert fname == cname, (fname, cname)
        assert cname in cf, "%s is not declared in funwave_gpu.h" % cname
        assert len(dummies) == cf[cname], "%s: %d Fortran arguments, %d in C" % (cname, len(dummies), cf[cname])
        missing = [d for d in dummies if d not in declared]
        assert not missing, "%s: arguments without a declaration: %s" % (cname, missing)
        seen.add(cname)
    unbound = sorted(set(cf) - seen)
    assert not unbound, "header functions without a Fortran interface: %s" % unbound


def test_status_constants_match_header():
    s = open(HDR).read()
    c = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(FW_(?:OK|ERR_\w+))\s+(-?\d+)", s)}
    f = {}
    for l in _fortran_lines():
        if "PARAMETER" in l.upper():
            for m in re.finditer(r"(FW_(?:OK|ERR_\w+))\s*=\s*(-?\d+)", l):
                f[m.group(1)] = int(m.group(2))
    assert f == c


def test_free_form_line_length():
    for k, raw in enumerate(open(F90).read().splitlines(), 1):
        assert len(raw) <= 132, "line %d has %d characters" % (k, len(raw))


def test_library_exports_every_bound_name(fw):
    L = fw.load_library()
    for _, cname, _, _ in _f_interfaces():
        assert hasattr(L, cname), cname
