"""The Fortran interface module (minisod2d_gb300/fortran/msod_capi.f90) against include/msod.h.

A Fortran host binds the C ABI through this module's ISO_C_BINDING interfaces.  No Fortran
compiler is available to build it, so its interfaces are parsed here and checked declaration by
declaration against the header: the same entry points, bind(C) names, argument counts and argument
kinds (scalars by value with the matching C kind, pointers as type(c_ptr) by value, pointer-to-
pointer outputs as type(c_ptr) by reference), the same return kinds and the same constants.  The
Python binding's signature table (capi.SIGNATURES) is checked against the same parse.
"""
import os
import re

from minisod2d_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "msod.h")
MODULE = os.path.join(ROOT, "minisod2d_gb300", "fortran", "msod_capi.f90")

SCALAR = {"int": "integer(c_int)", "float": "real(c_float)", "double": "real(c_double)",
          "size_t": "integer(c_size_t)", "int64_t": "integer(c_int64_t)", "uint64_t": "integer(c_int64_t)"}


def header_decls():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    out = {}
    for m in re.finditer(r"\n((?:const\s+)?(?:int|char)\s*\*?)\s*(msod_\w+)\s*\(([^;{]*?)\)\s*;", src):
        ret, name, params = m.group(1).strip(), m.group(2), m.group(3).strip()
        ps = [] if params in ("", "void") else [p.strip() for p in params.split(",")]
        types = []
        for p in ps:
            t = re.match(r"(.*?)([A-Za-z_]\w*)$", p).group(1).replace("const", "").strip()
            types.append(re.sub(r"\s+", "", t))
        out[name] = ("char*" if "char" in ret else "int", types)
    return out


def module_decls():
    src = open(MODULE).read()
    body = src.split("interface", 1)[1].rsplit("end interface", 1)[0]
    out = {}
    for m in re.finditer(r"\n\s*(integer\(c_int\)|type\(c_ptr\)) function (\w+)\((.*?)\)\s*bind\(C, name=\"(\w+)\"\)"
                         r"(.*?)end function (\w+)", body, re.S):
        ret, name, args, bname, decls, endname = m.groups()
        assert name == bname == endname, (name, bname, endname)
        arglist = [a.strip() for a in args.replace("&", " ").replace("\n", " ").split(",") if a.strip()]
        kinds = {}
        for d in re.finditer(r"\n\s*(integer\(\w+\)|real\(\w+\)|type\(c_ptr\))(, value)? :: (\w+)", decls):
            kinds[d.group(3)] = (d.group(1), bool(d.group(2)))
        out[name] = (ret, arglist, kinds, decls)
    return src, out


def expected(ctype):
    stars = ctype.count("*")
    if stars == 2:
        return ("type(c_ptr)", False)
    if stars == 1:
        return ("type(c_ptr)", True)
    return (SCALAR[ctype], True)


def test_module_matches_header():
    hdr = header_decls()
    src, mod = module_decls()
    assert len(hdr) >= 50
    assert set(mod) == set(hdr), sorted(set(mod) ^ set(hdr))
    for name, (cret, ctypes_) in hdr.items():
        ret, args, kinds, decls = mod[name]
        assert ret == ("type(c_ptr)" if cret == "char*" else "integer(c_int)"), name
        assert len(args) == len(ctypes_), name
        assert len({a.lower() for a in args}) == len(args), name  # Fortran names ignore case
        for a, ct in zip(args, ctypes_):
            assert kinds.get(a) == expected(ct), (name, a, ct, kinds.get(a))
        used = {k[0][k[0].index("(") + 1:-1] for k in kinds.values()} | {ret[ret.index("(") + 1:-1]}
        imp = re.search(r"import :: ([\w, ]+)", decls).group(1)
        assert used <= {x.strip() for x in imp.split(",")}, name


def test_module_constants_and_form():
    src = open(HEADER).read()
    consts = dict(re.findall(r"#define (MSOD_\w+) (\d+)", src))
    msrc, _ = module_decls()
    got = dict(re.findall(r"integer\(c_int\), parameter :: (MSOD_\w+) = (\d+)", msrc))
    assert got == consts
    for i, line in enumerate(msrc.splitlines(), 1):
        assert len(line) <= 132, "line %d longer than free-form Fortran allows" % i
        assert "\t" not in line, i


def test_python_binding_matches_header():
    hdr = header_decls()
    assert set(capi.SIGNATURES) == set(hdr), sorted(set(capi.SIGNATURES) ^ set(hdr))
    for name, (_, ctypes_) in hdr.items():
        assert len(capi.SIGNATURES[name]) == len(ctypes_), name
