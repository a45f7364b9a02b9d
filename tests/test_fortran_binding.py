"""The Fortran binding (fortran/examd_gpu_mod.f90) against the C header.

No Fortran compiler exists on this machine or on the GPU host, so the module
is checked by reading it: every entry point that include/examd_gb300.h
declares has exactly one bind(C, name=...) interface of the same name, with
the same number of arguments, and each argument and result is declared with
the ISO_C_BINDING kind and passing convention of its C type (by value for C
scalars, by reference or Type(c_ptr) for C pointers).  The bind(C) derived
types list the fields of examd_params, examd_box and examd_stats in the C
order with matching kinds.  The shim (fortran/examd_forces_gpu.f90) uses the
reference's own module and variable names (SRC/exaMD_module.f90:17,57-58;
user_func.f90:9,18) and calls only bound entry points.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "examd_gb300.h")
MOD = os.path.join(ROOT, "fortran", "examd_gpu_mod.f90")
SHIM = os.path.join(ROOT, "fortran", "examd_forces_gpu.f90")


def c_prototypes():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    src = re.sub(r"#.*", "", src)
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(examd_\w+)\s*\(([^)]*)\)\s*;", src):
        ret, name, args = m.group(1).strip(), m.group(2), m.group(3).strip()
        params = []
        if args and args != "void":
            for a in args.split(","):
                a = " ".join(a.split())
                if "[" in a:  # "const double L[3]": a pointer in the prototype
                    ty = a.split("[")[0].rsplit(" ", 1)[0] + "*"
                else:
                    ty = re.match(r"(.*?)(\w+)$", a).group(1).strip()
                params.append(ty.replace(" *", "*").strip())
        out[name] = (ret, params)
    return out


def c_structs():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct (examd_\w+) \{(.*?)\}", src, flags=re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            ty, names = decl.split(" ", 1)
            for nm in names.split(","):
                nm = nm.strip()
                arr = re.search(r"\[(.*)\]", nm)
                fields.append((re.sub(r"\[.*\]", "", nm), ty, bool(arr)))
        out[m.group(1)] = fields
    return out


def fortran_lines(path):
    """Source lines with comments removed and & continuations joined."""
    lines, cur = [], ""
    for raw in open(path):
        ln = raw.split("!")[0].rstrip()
        if not ln.strip():
            continue
        if cur:
            ln = cur + " " + ln.strip().lstrip("&").strip()
            cur = ""
        if ln.endswith("&"):
            cur = ln[:-1].rstrip()
            continue
        lines.append(ln.strip())
    return lines


def fortran_interfaces():
    lines = fortran_lines(MOD)
    out, i = {}, 0
    head = re.compile(r"(?:(Integer\(c_int\)|Type\(c_ptr\))\s+)?(Subroutine|Function)\s+(\w+)\s*\(([^)]*)\)\s*"
                      r"bind\(C,\s*name=\"(\w+)\"\)", re.I)
    while i < len(lines):
        m = head.match(lines[i])
        if not m:
            i += 1
            continue
        result, kind, fname, args, cname = m.groups()
        dummies = [a.strip() for a in args.split(",") if a.strip()]
        decls = {}
        i += 1
        while not re.match(r"End\s+(Subroutine|Function)", lines[i], re.I):
            d = re.match(r"(.+?)::\s*(.+)$", lines[i])
            if d and not lines[i].lower().startswith("import"):
                attrs = [x.strip() for x in d.group(1).split(",")]
                for nm in re.split(r",\s*(?![^()]*\))", d.group(2)):
                    base = re.match(r"(\w+)", nm.strip()).group(1)
                    decls[base] = (attrs, "(" in nm)
            i += 1
        out[cname] = (fname, kind, result, dummies, decls)
        i += 1
    return out


SCALAR = {"int": "integer(c_int)", "int64_t": "integer(c_int64_t)", "uint64_t": "integer(c_int64_t)",
          "double": "real(c_double)"}
POINTEE = {"double": "real(c_double)", "int": "integer(c_int)", "int64_t": "integer(c_int64_t)",
           "char": "character(kind=c_char)", "signed char": "integer(c_signed_char)",
           "unsigned char": "integer(c_signed_char)", "examd_params": "type(examd_params)",
           "examd_box": "type(examd_box)", "examd_stats": "type(examd_stats)", "void*": "type(c_ptr)",
           "examd_ctx*": "type(c_ptr)"}


def kind_of(attrs):
    return attrs[0].replace(" ", "").lower()


def test_every_entry_point_is_bound_once():
    c = c_prototypes()
    f = fortran_interfaces()
    assert len(c) >= 25
    assert sorted(c) == sorted(f), (set(c) ^ set(f))
    for cname, (fname, *_rest) in f.items():
        assert fname == cname


@pytest.mark.parametrize("name", sorted(c_prototypes()))
def test_arguments_match_the_c_prototype(name):
    ret, params = c_prototypes()[name]
    fname, kind, result, dummies, decls = fortran_interfaces()[name]
    # result: int -> Integer(c_int) Function, void -> Subroutine, const char * -> Type(c_ptr) Function
    if ret == "void":
        assert kind.lower() == "subroutine"
    elif ret == "int":
        assert kind.lower() == "function" and result.lower() == "integer(c_int)"
    else:
        assert "char" in ret and kind.lower() == "function" and result.lower() == "type(c_ptr)"
    assert len(dummies) == len(params), (dummies, params)
    for d, ct in zip(dummies, params):
        attrs, is_array = decls[d]
        fk = kind_of(attrs)
        by_value = any(a.lower() == "value" for a in attrs)
        ct_plain = ct.replace("const ", "").strip()
        if "*" not in ct_plain:  # C scalar by value
            assert by_value and fk == SCALAR[ct_plain], (d, ct, attrs)
            continue
        pointee = ct_plain[:-1].strip()
        if ct_plain.endswith("**"):  # examd_ctx **out
            assert fk == "type(c_ptr)" and not by_value, (d, ct, attrs)
        elif fk == "type(c_ptr)" and by_value:  # nullable pointer passed as c_ptr
            pass
        else:
            assert not by_value, (d, ct, attrs)
            want = POINTEE.get(pointee, POINTEE.get(ct_plain))
            assert fk == want, (d, ct, attrs)


def test_derived_types_match_the_c_structs():
    structs = c_structs()
    lines = fortran_lines(MOD)
    ftypes, cur = {}, None
    for ln in lines:
        m = re.match(r"Type,\s*bind\(C\)\s*::\s*(\w+)", ln, re.I)
        if m:
            cur = m.group(1)
            ftypes[cur] = []
            continue
        if cur and re.match(r"End Type", ln, re.I):
            cur = None
            continue
        if cur:
            ty, names = ln.split("::")
            for nm in re.split(r",\s*(?![^()]*\))", names):
                ftypes[cur].append((re.match(r"(\w+)", nm.strip()).group(1), ty.strip().lower().replace(" ", ""),
                                    "(" in nm))
    ctof = {"int": "integer(c_int)", "double": "real(c_double)", "int64_t": "integer(c_int64_t)"}
    for name in ("examd_params", "examd_box", "examd_stats"):
        cf, ff = structs[name], ftypes[name]
        assert [x[0] for x in cf] == [x[0] for x in ff], name
        for (cn, cty, carr), (fn, fty, farr) in zip(cf, ff):
            assert ctof[cty] == fty and carr == farr, (name, cn)


def test_status_codes_match_the_header():
    src = open(HEADER).read()
    codes = dict(re.findall(r"#define (EXAMD_(?:OK|ERR_\w+))\s+(\d+)", src))
    mod = open(MOD).read()
    for name, val in codes.items():
        assert re.search(rf"{name} = {val}\b", mod), name


def test_shim_uses_the_reference_names_and_bound_entry_points():
    shim = open(SHIM).read()
    code = "\n".join(fortran_lines(SHIM))
    assert re.search(r"^Use exaMD_mod$", code, re.M)           # SRC/exaMD_module.f90:17
    assert re.search(r"^Use user_func_mod, Only: prmvdw$", code, re.M)  # user_func.f90:9,18
    for sym in ("locblocks", "nblocks_loc", "globalbox", "COMM_EXAMD", "grid(i,j,k)%posn", "grid(i,j,k)%forces"):
        assert sym in code, sym
    for bad in ("exaMD_module", "total_atoms"):
        assert bad not in code, bad
    bound = set(fortran_interfaces())
    called = set(re.findall(r"\b(examd_[a-z_]+)\s*\(", code)) - {"examd_params", "examd_box", "examd_forces_gpu_mod"}
    assert called and called <= bound, called - bound
    assert "forces(:, 1:na) = grid(i,j,k)%forces(:, 1:na) +" in shim.replace("&\n            ", "")
