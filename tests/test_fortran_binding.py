"""The Fortran side of the boundary (flexi_gb300/fortran/mod_dg_gpu.f90) against the C header (include/flexi_gpu.h).

No Fortran compiler exists on these machines, so the binding is checked by reading both files: every C function has one
BIND(C,NAME=...) interface with the same number and order of arguments, each argument with the Fortran declaration that
passes what the C prototype expects (VALUE for scalars passed by value, by reference for pointers, TYPE(C_PTR) for handles
and opaque pointers, OPTIONAL only where the C side accepts NULL), the BIND(C) derived types have the C structs' fields
in order with matching types, and the shim procedures use no name they neither declare nor import (IMPLICIT NONE)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "flexi_gpu.h")
F90 = os.path.join(ROOT, "flexi_gb300", "fortran", "mod_dg_gpu.f90")


def c_prototypes():
    h = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for ret, name, args in re.findall(r"^\s*((?:const\s+)?[A-Za-z_][A-Za-z_0-9 ]*\**)\s*\b(fg_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", h, flags=re.M):
        args = " ".join(args.split())
        lst = [] if args in ("", "void") else [a.strip() for a in args.split(",")]
        out[name] = (" ".join(ret.split()), lst)
    return out


def c_structs():
    h = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for body, name in re.findall(r"typedef struct \w+ \{(.*?)\} (\w+);", h, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            parts = [p.strip() for p in decl.split(",")]
            m = re.match(r"^(.+?)\s*(\**)\s*(\w+)\s*(?:\[(\d+)\])?$", parts[0])
            assert m, decl
            base = m.group(1).strip()
            items = [(m.group(2), m.group(3), m.group(4))]
            for p in parts[1:]:
                mm = re.match(r"^(\**)\s*(\w+)\s*(?:\[(\d+)\])?$", p)
                items.append(mm.groups())
            for ptr, nm, dim in items:
                fields.append((nm, base + ptr, int(dim) if dim else 0))
        out[name] = fields
    return out


def fortran_source():
    lines = []
    for ln in open(F90).read().splitlines():
        ln = ln.split("!")[0] if "'" not in ln else re.sub(r"!(?=[^']*$).*", "", ln)
        lines.append(ln)
    # join continuation lines
    text = "\n".join(lines)
    text = re.sub(r"&\s*\n\s*&?", " ", text)
    return text


def fortran_interfaces():
    text = fortran_source()
    block = text[text.index("INTERFACE"):text.index("END INTERFACE")]
    out = {}
    for m in re.finditer(r"(INTEGER\(C_INT\)|INTEGER\(C_LONG_LONG\)|INTEGER\(C_SIZE_T\)|TYPE\(C_PTR\)) FUNCTION (\w+)\(([^)]*)\)\s*"
                         r"BIND\(C,NAME='(\w+)'\)(.*?)END FUNCTION", block, flags=re.S):
        ret, fname, args, cname, body = m.groups()
        argnames = [a.strip() for a in args.split(",") if a.strip()]
        decls = {}
        for stmt in re.split(r"[;\n]", body):
            stmt = stmt.strip()
            if not stmt or stmt == "IMPORT":
                continue
            if stmt.startswith("IMPORT"):
                stmt = stmt[len("IMPORT"):].strip()
            typ, names = stmt.split("::")
            attrs = [a.strip() for a in re.split(r",(?![^()]*\))", typ)]
            for nm in names.split(","):
                nm = nm.strip()
                arr = "(*)" in nm or re.search(r"\(\d+\)", nm) is not None
                decls[re.sub(r"\(.*\)", "", nm)] = (attrs[0], set(attrs[1:]), arr)
        if cname.startswith("fg_"):  # the module also binds the C library's strlen for messages
            out[cname] = (ret, fname, argnames, decls)
    return out


# C type of an argument -> predicate on the Fortran declaration (base type, attributes, is-array)
def expected(ctype, nullable):
    t = ctype.replace("const ", "").strip()
    base = t.rstrip("*").strip()
    ptr = t.count("*")
    if ptr == 0:
        return {"int": ("INTEGER(C_INT)", True), "double": ("REAL(C_DOUBLE)", True)}[base]
    if ptr == 2 or base == "void":
        return ("TYPE(C_PTR)", ptr == 1)  # void*: opaque pointer by value; T**: a C_PTR written by the library
    if base in ("fg_handle",):
        return ("TYPE(C_PTR)", True)
    m = {"int": "INTEGER(C_INT)", "double": "REAL(C_DOUBLE)", "long long": "INTEGER(C_LONG_LONG)", "char": "CHARACTER(KIND=C_CHAR)",
         "fg_config": "TYPE(fg_config)", "fg_timedisc_state": "TYPE(fg_timedisc_state)", "fg_device_mesh": "TYPE(fg_device_mesh)"}[base]
    return (m, False)


# device addresses (caller-owned device memory): opaque pointers passed by value
DEVICE_PTRS = {"fg_time_derivative_noalloc": {"U", "Ut"}}

# arguments the C side documents as nullable (NULL accepted): only these may be OPTIONAL in Fortran
NULLABLE = {"fg_build_mesh": {"ElemInst"}, "fg_build_mesh_mortar": {"ElemInst", "Mortars"}, "fg_hopr_read": {"BCNames", "Mortars"},
            "fg_time_derivative": {"Ut"}, "fg_run": {"t"}, "fg_get_gradients": {"gx", "gy", "gz"}, "fg_set_elem_mu_scale": {"scale"},
            "fg_vjp_time_derivative": {"muScaleBar"}, "fg_adjoint_reverse": {"Ubar0", "muScaleBar", "forceBar"},
            "fg_set_body_force_field": {"F"}, "fg_wall_shear": {"dJdU"}, "fg_autotune": {"report"}}


def test_every_c_function_is_bound():
    c, f = c_prototypes(), fortran_interfaces()
    assert len(c) >= 50
    assert set(c) == set(f), (set(c) ^ set(f))
    for name, (ret, fname, _, _) in f.items():
        assert fname == name


@pytest.mark.parametrize("name", sorted(c_prototypes()))
def test_interface_matches_prototype(name):
    cret, cargs = c_prototypes()[name]
    fret, _, fargs, decls = fortran_interfaces()[name]
    assert {"int": "INTEGER(C_INT)", "long long": "INTEGER(C_LONG_LONG)", "const char*": "TYPE(C_PTR)"}[cret] == fret
    assert len(cargs) == len(fargs), (cargs, fargs)
    for ca, fa in zip(cargs, fargs):
        ctype = " ".join(ca.split()[:-1]) + "*" * ca.split()[-1].count("*")
        cname = ca.split()[-1].replace("*", "")
        assert fa in decls, (name, fa)
        ftype, attrs, _ = decls[fa]
        if cname in DEVICE_PTRS.get(name, ()):
            want_type, want_value = "TYPE(C_PTR)", True
        else:
            want_type, want_value = expected(ctype, cname in NULLABLE.get(name, ()))
        assert ftype == want_type, (name, ca, ftype)
        assert ("VALUE" in attrs) == want_value, (name, ca, attrs)
        if "OPTIONAL" in attrs:
            assert cname in NULLABLE.get(name, ()), (name, ca, "OPTIONAL where C does not accept NULL")
        assert fa.lower() == cname.lower() or name in ("fg_create", "fg_hopr_sizes", "fg_get_sizes", "fg_get_mesh_array",
                                                       "fg_get_side_to_elem", "fg_get_timedisc_state", "fg_debug_array",
                                                       "fg_autotune_choice", "fg_get_config"), (name, ca, fa)


def test_derived_types_match_structs():
    text = fortran_source()
    structs = c_structs()
    ctypes_map = {"int": "INTEGER(C_INT)", "double": "REAL(C_DOUBLE)", "long long": "INTEGER(C_LONG_LONG)"}
    for sname, fields in structs.items():
        m = re.search(r"TYPE, BIND\(C\), PUBLIC :: %s\n(.*?)END TYPE %s" % (sname, sname), text, flags=re.S)
        assert m, sname
        fdecl = []
        for ln in m.group(1).splitlines():
            if "::" not in ln:
                continue
            typ, names = ln.split("::")
            for nm in names.split(","):
                nm = nm.strip()
                dim = re.search(r"\((\d+)\)", nm)
                fdecl.append((re.sub(r"\(.*\)", "", nm), typ.strip(), int(dim.group(1)) if dim else 0))
        assert len(fdecl) == len(fields), (sname, fdecl, fields)
        for (fn, ft, fd), (cn, ct, cd) in zip(fdecl, fields):
            want = "TYPE(C_PTR)" if ct.endswith("*") else ctypes_map[ct.replace("const ", "")]
            assert fn.lower() == cn.lower() and ft == want and fd == cd, (sname, (fn, ft, fd), (cn, ct, cd))


def test_error_codes_match():
    h = open(HEADER).read()
    text = fortran_source()
    for name, val in re.findall(r"#define (FG_OK|FG_ERR_\w+) (\d+)", h):
        assert re.search(r"\b%s=%s\b" % (name, val), text), name


KEYWORDS = set("""SUBROUTINE FUNCTION END USE ONLY IMPLICIT NONE INTEGER REAL LOGICAL CHARACTER TYPE INTENT IN OUT INOUT IF THEN ELSE
RETURN CALL SELECT CASE DEFAULT DO RESULT KIND LEN POINTER VALUE OPTIONAL PARAMETER TRUE FALSE NOT EQ NE GT LT GE LE AND OR
TRIM INT MIN MAX MERGE HUGE C_ASSOCIATED C_F_POINTER C_NULL_PTR C_INT C_DOUBLE C_PTR C_CHAR C_SIZE_T C_LONG_LONG C_LOC
IntInfo""".split())


def test_shim_names_are_declared():
    text = fortran_source()
    module = text[:text.index("CONTAINS")]
    body = text[text.index("CONTAINS") + len("CONTAINS"):]
    module_names = set(re.findall(r"\b(fg_\w+|FG_\w+|gpu|useGPU|c_strlen)\b", module))
    procs = re.findall(r"\n(?:SUBROUTINE|FUNCTION) (\w+)\((.*?)\)(.*?)\nEND (?:SUBROUTINE|FUNCTION) \1", body, flags=re.S)
    assert {p[0] for p in procs} >= {"InitDG_GPU", "DGTimeDerivative_GPU", "TimeStepByLSERKW2_GPU", "CalcTimeStep_GPU",
                                     "TimeDiscSteps_GPU", "GetState_GPU", "FinalizeDG_GPU"}
    proc_names = {p[0] for p in procs}
    for name, args, src in procs:
        src = re.sub(r"'[^']*'", "''", src)
        lines = [ln for ln in src.splitlines() if not ln.strip().startswith("#")]
        declared = set(a.strip() for a in args.split(",") if a.strip())
        m = re.search(r"RESULT\((\w+)\)", src)
        if m:
            declared.add(m.group(1))
        used = set()
        for ln in lines:
            s = ln.strip()
            if s.startswith("USE "):
                if "ONLY:" in s:
                    declared |= {x.strip() for x in s.split("ONLY:")[1].split(",")}
                continue
            if "::" in s and re.match(r"(INTEGER|REAL|LOGICAL|CHARACTER|TYPE)\b", s):
                declared |= {re.sub(r"\(.*", "", x.strip()) for x in re.split(r",(?![^()]*\))", s.split("::")[1])}
                continue
            s = re.sub(r"\.\w+\.", " ", s)           # .EQ., .TRUE., ...
            s = re.sub(r"%\w+", "", s)              # components
            s = re.sub(r"\b\d+(_C_INT)?\b", " ", s)  # literals
            used |= set(re.findall(r"\b[A-Za-z_]\w*\b", s))
        undeclared = {u for u in used if u not in declared and u not in module_names and u not in proc_names and u not in KEYWORDS
                      and not u.startswith("PP_") and u not in ("__STAMP__", "SPLIT_DG")}
        assert not undeclared, (name, sorted(undeclared))


def test_free_form_line_length():
    """Free-form Fortran lines stay within the standard's 132 characters (no compiler flag needed)."""
    long_lines = [(i + 1, len(ln)) for i, ln in enumerate(open(F90).read().splitlines()) if len(ln) > 132]
    assert not long_lines, long_lines
