"""The Fortran interface module (fib_md_gb300/fortran/fibmd_gpu_mod.f90)
against the C header it binds. No Fortran compiler is available, so the
module is checked by reading it: every bind(C) interface names a function
of include/fibmd_gpu.h with the same number of arguments, each argument
passed the same way (by value or by reference) with a matching C type;
every entry point but the device-pointer one is bound; and
type(fibmd_params) and type(fibmd_replica) list the C structs' fields in
order with the same types and array lengths (bind(C) derived types take the
C layout)."""
from __future__ import annotations

import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
F90 = ROOT / "fib_md_gb300" / "fortran" / "fibmd_gpu_mod.f90"
HDR = ROOT / "include" / "fibmd_gpu.h"


def _strip_c(text):
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def _c_functions():
    out = {}
    for m in re.finditer(r"\b(int|void)\s+(fibmd_gpu_\w+)\s*\(([^)]*)\)\s*;", _strip_c(HDR.read_text())):
        args = [a.strip() for a in " ".join(m.group(3).split()).split(",")]
        out[m.group(2)] = (m.group(1), [] if args == ["void"] else args)
    return out


def _c_kind(arg):
    """(base, by_reference) of a C parameter declaration."""
    a = arg.replace("const ", "")
    ref = "*" in a or "[" in a
    for base in ("fibmd_params", "fibmd_replica", "fibmd_ctx", "long long", "uint32_t", "double",
                 "char", "int"):
        if re.search(r"\b" + base + r"\b", a):
            if base == "fibmd_ctx":
                return ("ctxptr", a.count("*") == 2)
            return (base, ref)
    raise AssertionError(arg)


def _f_interfaces():
    src = F90.read_text()
    body = src[src.index("interface"):src.index("end interface")]
    out = {}
    for m in re.finditer(
            r"(integer\(c_int\)\s+function|subroutine)\s+(\w+)\s*\(([^)]*)\)\s*&?\s*bind\(C\)(.*?)end\s+(?:function|subroutine)",
            body, flags=re.S):
        names = [a.strip() for a in m.group(3).replace("&", " ").split(",") if a.strip()]
        decls = {}
        for line in m.group(4).splitlines():
            line = line.strip()
            if "::" not in line:
                continue
            spec, vars_ = line.split("::")
            for v in vars_.split(","):
                v = v.strip()
                vn = v.split("(")[0].strip()
                decls[vn] = (spec.strip(), "(" in v)
        out[m.group(2)] = ("int" if m.group(1).startswith("integer") else "void", names, decls)
    return out


def _f_kind(spec, is_array):
    by_value = "value" in spec
    if spec.startswith("type(c_ptr)"):
        return ("ctxptr", not by_value)
    if spec.startswith("type(fibmd_params)"):
        return ("fibmd_params", True)
    if spec.startswith("type(fibmd_replica)"):
        return ("fibmd_replica", True)
    kinds = {"c_int)": "int", "c_int32_t)": "uint32_t", "c_double)": "double",
             "c_long_long)": "long long", "kind=c_char)": "char"}
    for k, base in kinds.items():
        if k in spec:
            return (base, not by_value)
    raise AssertionError(spec)


def test_bindings_match_the_header():
    cf = _c_functions()
    ff = _f_interfaces()
    assert len(ff) >= 33
    # every entry point is bound but the one taking device pointers
    # (fibmd_gpu_stream returns a pointer and is not matched above)
    assert set(cf) - set(ff) == {"fibmd_gpu_force_noalloc"}
    for name, (ret, args, decls) in ff.items():
        assert name in cf, name
        cret, cargs = cf[name]
        assert ret == cret, name
        assert len(args) == len(cargs), name
        for a, ca in zip(args, cargs):
            assert a in decls, (name, a)
            assert _f_kind(*decls[a]) == _c_kind(ca), (name, a, decls[a], ca)


def _c_struct_fields(name="fibmd_params"):
    s = _strip_c(HDR.read_text())
    head = "typedef struct %s {" % name
    body = s[s.index(head) + len(head):s.index("} %s;" % name)]
    fields = []
    for decl in body.split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        base, rest = decl.split(" ", 1)
        for v in rest.split(","):
            v = v.strip()
            m = re.match(r"(\w+)(?:\[(\d+)\])?", v)
            fields.append((m.group(1).lower(), base, int(m.group(2) or 1)))
    return fields


def _f_struct_fields(name="fibmd_params"):
    src = F90.read_text()
    body = src[src.index("type, bind(C) :: " + name):src.index("end type " + name)]
    fields = []
    for line in body.splitlines()[1:]:
        if "::" not in line:
            continue
        spec, vars_ = line.split("::")
        base = "int" if "c_int" in spec else "double"
        for v in vars_.split(","):
            m = re.match(r"\s*(\w+)(?:\((\d+)\))?", v)
            fields.append((m.group(1).lower(), base, int(m.group(2) or 1)))
    return fields


@pytest.mark.parametrize("name", ["fibmd_params", "fibmd_replica"])
def test_derived_types_match_the_structs(name):
    assert _f_struct_fields(name) == _c_struct_fields(name)
