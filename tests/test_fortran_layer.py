"""The Fortran drop-in layer (wtb_gb300/fortran), read as text: no Fortran compiler exists in the build image.

* module_bse.F90 and module_slepc_solver.F90 keep every public procedure of the reference's module_bse and
  module_slepc_solver with the same kind, result type, dummy-argument names in the same order, and each dummy's
  type and rank (tests/golden/reference_interfaces.json, recorded from the reference's sources by
  tests/golden/make_interfaces.py); every module_bse procedure main.F90 calls is there.
* The wtb_gpu_* versions of eigsys, hlm, optsp, optdiel, slepc_solver and the nine potentials keep their
  reference argument lists the same way.
* The bind(C) derived types have the fields, types and byte offsets of the C structs in include/wtb_gpu.h.
* Every bind(C) interface names an entry point include/wtb_gpu.h declares, with as many arguments, each passed
  by value exactly where the C parameter is not a pointer.
* The sources are well formed at the level a text check can see: free-form lines within 132 characters, every
  module, procedure, interface, type, do, select and if-then block closed.
"""
import ctypes
import json
import os
import re

import pytest

from tests.golden.fortran_decls import logical_lines, procedures

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FORT = os.path.join(ROOT, "wtb_gb300", "fortran")
REF = json.load(open(os.path.join(ROOT, "tests", "golden", "reference_interfaces.json")))
TWINS = {"eigsys": "wtb_gpu_eigsys", "hlm": "wtb_gpu_hlm", "optsp": "wtb_gpu_optsp", "optdiel": "wtb_gpu_optdiel",
         "slepc_solver": "wtb_gpu_slepc_solver", "v2dk": "wtb_gpu_v2dk", "vcoul": "wtb_gpu_vcoul",
         "v3diel": "wtb_gpu_v3diel", "v2dt": "wtb_gpu_v2dt", "v0dt": "wtb_gpu_v0dt", "v2dt2": "wtb_gpu_v2dt2",
         "v2drk": "wtb_gpu_v2drk", "v2dohono": "wtb_gpu_v2dohono", "v1dt": "wtb_gpu_v1dt"}


def src(name):
    return open(os.path.join(FORT, name)).read()


def test_dropin_modules_keep_the_reference_interfaces():
    ours = {}
    for f in ("module_bse.F90", "module_slepc_solver.F90"):
        ours.update(procedures(src(f)))
    assert re.search(r"^\s*module\s+module_bse\s*$", src("module_bse.F90"), re.M | re.I)
    assert re.search(r"^\s*module\s+module_slepc_solver\s*$", src("module_slepc_solver.F90"), re.M | re.I)
    checked = 0
    for name, ref in REF["procedures"].items():
        if ref["module"] not in ("module_bse", "module_slepc_solver"):
            continue
        assert name in ours, name
        got = ours[name]
        assert got["kind"] == ref["kind"] and got["result"] == ref["result"], name
        assert got["args"] == ref["args"], (name, got["args"], ref["args"])
        for a in ref["args"]:
            assert got["types"].get(a) == ref["types"][a], (name, a, got["types"].get(a), ref["types"][a])
        checked += 1
    assert checked == 21
    for name in REF["main_calls"]:
        assert name in ours, name
    # the module variables of the reference's module_bse
    text = src("module_bse.F90").lower()
    for v in ("dimbse", "hbse(:,:)", "ws(:)", "he(:,:)", "ltest", "ngkpt", "kpt(:,:)"):
        assert v in text, v


def test_gpu_versions_of_the_scalar_routines_keep_their_argument_lists():
    ours = procedures(src("wtb_gpu_iface.F90"))
    for ref_name, twin in TWINS.items():
        ref = REF["procedures"][ref_name]
        got = ours[twin]
        assert got["kind"] == ref["kind"] and got["result"] == ref["result"], ref_name
        assert got["args"] == ref["args"], (ref_name, got["args"], ref["args"])
        for a in ref["args"]:
            # type and rank; the reference's assumed-size (*) and explicit bounds are the same for a caller
            assert got["types"][a][:2] == ref["types"][a][:2], (ref_name, a, got["types"][a], ref["types"][a])


# ------------------------------------------------------------------------------------------- bind(C) layer
_CTYPES = {"int": ctypes.c_int, "double": ctypes.c_double, "float": ctypes.c_float}
_FTYPES = {"integer(c_int)": ctypes.c_int, "real(c_double)": ctypes.c_double, "real(c_float)": ctypes.c_float}


def c_struct_fields(header, name):
    """Fields of `typedef struct [tag] {...} name;` from the header: [(field, ctype)]."""
    text = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    m = re.search(r"typedef\s+struct\s*\w*\s*\{([^{}]*)\}\s*" + name + r"\s*;", text)
    assert m, name
    fields = []
    for decl in m.group(1).split(";"):
        decl = decl.strip()
        if not decl:
            continue
        base, rest = decl.split(None, 1)
        for item in rest.split(","):
            item = item.strip()
            mm = re.match(r"(\w+)(?:\[(\d+)\])?", item)
            t = _CTYPES[base]
            fields.append((mm.group(1), t * int(mm.group(2)) if mm.group(2) else t))
    return fields


def f_type_fields(text, name):
    m = re.search(r"type\s*,\s*bind\(C\)\s*::\s*" + name + r"\s*\n(.*?)end\s+type", text, re.S | re.I)
    assert m, name
    fields = []
    for ln in logical_lines(m.group(1)):
        if "::" not in ln:
            continue
        t, names = ln.split("::")
        t = re.sub(r"\s+", "", t.lower())
        for item in names.split(","):
            mm = re.match(r"\s*(\w+)\s*(?:\((\d+)\))?", item)
            ct = _FTYPES[t]
            fields.append((mm.group(1), ct * int(mm.group(2)) if mm.group(2) else ct))
    return fields


def layout(fields):
    S = type("S", (ctypes.Structure,), {"_fields_": fields})
    return [(n, getattr(S, n).offset, getattr(S, n).size) for n, _ in fields], ctypes.sizeof(S)


@pytest.mark.parametrize("fname,cname", [("wtb_bse_params_t", "wtb_bse_params"), ("wtb_timings_t", "wtb_timings"),
                                         ("wtb_temp_params_t", "wtb_temp_params")])
def test_bind_c_types_match_the_header(fname, cname):
    header = open(os.path.join(ROOT, "include", "wtb_gpu.h")).read()
    cf = c_struct_fields(header, cname)
    ff = f_type_fields(src("wtb_gpu_iface.F90"), fname)
    assert [n for n, _ in ff] == [n for n, _ in cf]
    assert layout(ff) == layout(cf)


def c_prototypes(header):
    text = re.sub(r"/\*.*?\*/", "", header, flags=re.S)
    protos = {}
    for m in re.finditer(r"^\s*(?:const\s+)?[\w ]+?\**\s*\**(wtb_\w+)\s*\(([^)]*)\)\s*;", text, re.M):
        params = [p.strip() for p in m.group(2).replace("\n", " ").split(",") if p.strip() and p.strip() != "void"]
        protos[m.group(1)] = ["*" in p or "[" in p for p in params]
    return protos


def f_interfaces(text):
    out = {}
    body = re.search(r"^\s*interface\s*$(.*?)^\s*end\s+interface", text, re.S | re.M | re.I).group(1)
    for blk in re.finditer(r"function\s+(\w+)\s*\(([^)]*)\)\s*&?\s*(?:&\s*)?bind\(C,\s*name=\"(\w+)\"\)(.*?)end\s+function",
                           body, re.S | re.I):
        args = [a.strip().lower() for a in blk.group(2).replace("&", " ").split(",") if a.strip()]
        by_value = {a: False for a in args}
        for ln in logical_lines(blk.group(4)):
            if "::" not in ln:
                continue
            t, names = ln.split("::")
            # by value, and not a C pointer passed by value (type(c_ptr), value)
            val = bool(re.search(r",\s*value\b", t, re.I)) and not re.match(r"\s*type\(c_ptr\)", t, re.I)
            for item in names.split(","):
                nm = re.match(r"\s*(\w+)", item).group(1).lower()
                if nm in by_value:
                    by_value[nm] = val
        out[blk.group(3)] = [not by_value[a] for a in args]
    return out


def test_bind_c_interfaces_match_the_header_prototypes():
    protos = c_prototypes(open(os.path.join(ROOT, "include", "wtb_gpu.h")).read())
    ifs = f_interfaces(src("wtb_gpu_iface.F90"))
    assert len(ifs) >= 38
    for cname, f_ptr in ifs.items():
        assert cname in protos, cname
        # a Fortran dummy without VALUE is passed by reference: the C parameter must be a pointer, and back
        assert f_ptr == protos[cname], (cname, f_ptr, protos[cname])


# ------------------------------------------------------------------------------------------- well-formedness
@pytest.mark.parametrize("name", ["wtb_gpu_iface.F90", "module_bse.F90", "module_slepc_solver.F90"])
def test_fortran_sources_are_well_formed(name):
    text = src(name)
    for i, ln in enumerate(text.splitlines(), 1):
        assert len(ln) <= 132, (name, i, len(ln))
    lines = [ln.strip().lower() for ln in logical_lines(text) if ln.strip()]

    def count(pat):
        return sum(1 for ln in lines if re.match(pat, ln))

    assert count(r"^module\s+\w+$") == count(r"^end\s+module\b") == 1
    assert count(r"^(?:(?:complex\(8\)|real\(8\)|integer(?:\(c_int\))?|double\s+precision|type\(c_ptr\))\s+)?"
                 r"function\s+\w+") == count(r"^end\s+function\b")
    assert count(r"^subroutine\s+\w+") == count(r"^end\s+subroutine\b")
    assert count(r"^interface\s*$") == count(r"^end\s+interface\b")
    assert count(r"^type\s*(?:,\s*bind\(c\))?\s*::") == count(r"^end\s+type\b")
    assert count(r"^do\b") == count(r"^end\s*do\b")
    assert count(r"^select\s+case\b") == count(r"^end\s+select\b")
    assert count(r"^(?:else\s+)?if\s*\(.*\)\s*then$") - count(r"^else\s+if\s*\(.*\)\s*then$") == count(r"^end\s*if\b")
    # every name a procedure passes to c_wtb_* as a C string is NUL-terminated
    for m in re.finditer(r"wtb_gpu_check\(c_wtb_write_\w+\(([^,]+),", text):
        arg = m.group(1)
        assert "wtb_cstr(" in arg or "c_null_char" in arg, arg
