"""The Fortran interface module (include/galaexi_gb300.f90) against the C header and the library.

No Fortran compiler exists in this image, so the module is checked by reading it: every function the C
header declares has exactly one BIND(C) procedure with the same number of arguments, exported by
libgalaexi_gb300.so; the BIND(C) dg_config type lists the C struct's fields in the same order with
matching kinds; the integer parameters equal the header's #define constants, all of which are
present; and every line fits Fortran's 132-character free-form limit.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "include", "galaexi_gb300.f90")
HDR = os.path.join(ROOT, "include", "galaexi_gb300.h")


def _fortran_statements():
    """Free-form statements with continuation lines joined and comments dropped."""
    out, cur = [], ""
    for line in open(F90):
        code = line.split("!", 1)[0].rstrip()
        if not code.strip():
            continue
        if code.endswith("&"):
            cur += code[:-1] + " "
            continue
        out.append((cur + code).strip())
        cur = ""
    return out


def _c_declarations():
    text = re.sub(r"/\*.*?\*/", " ", open(HDR).read(), flags=re.S)
    decls = {}
    for m in re.finditer(r"\b([A-Za-z_][\w\s\*]*?)\b(dg_\w+)\s*\(([^;{}]*?)\)\s*;", text):
        args = [a.strip() for a in m.group(3).split(",") if a.strip() and a.strip() != "void"]
        decls[m.group(2)] = args
    return text, decls


def test_bind_c_procedures_match_header_and_exports():
    from galaexi_gb300 import _native as nat
    lib = nat.lib()
    _, decls = _c_declarations()
    procs = []
    for st in _fortran_statements():
        m = re.search(r"(?:FUNCTION|SUBROUTINE)\s+(\w+)\s*\(([^)]*)\)\s*BIND\s*\(\s*C\s*,\s*NAME\s*=\s*'(\w+)'\s*\)",
                      st, flags=re.I)
        if m:
            args = [a.strip() for a in m.group(2).split(",") if a.strip()]
            procs.append((m.group(1), args, m.group(3)))
    # every entry point of the header has a binding, and no name is bound twice
    assert sorted(c for _, _, c in procs) == sorted(decls)
    for fname, args, cname in procs:
        assert fname.lower() == cname.lower()
        assert cname in decls, cname
        assert len(args) == len(decls[cname]), (cname, args, decls[cname])
        assert hasattr(lib, cname), cname


def test_config_type_matches_c_struct():
    text, _ = _c_declarations()
    body = re.search(r"typedef struct dg_config\s*\{(.*?)\}\s*dg_config;", text, flags=re.S).group(1)
    c_fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        for nm in names.split(","):
            nm = nm.strip()
            m = re.match(r"(\w+)(?:\[(\d+)\])?$", nm)
            c_fields.append((m.group(1).lower(), ctype, int(m.group(2) or 1)))
    f_fields = []
    in_type = False
    for st in _fortran_statements():
        if re.match(r"TYPE\s*,\s*BIND\s*\(\s*C\s*\)\s*::\s*dg_config", st, flags=re.I):
            in_type = True
            continue
        if in_type and re.match(r"END\s+TYPE", st, flags=re.I):
            break
        if in_type:
            kind, names = st.split("::")
            for nm in names.split(","):
                m = re.match(r"\s*(\w+)(?:\((\d+)\))?\s*$", nm)
                f_fields.append((m.group(1).lower(), kind.strip().upper(), int(m.group(2) or 1)))
    assert [f[0] for f in f_fields] == [c[0] for c in c_fields]
    kinds = {"int": "INTEGER(C_INT)", "double": "REAL(C_DOUBLE)"}
    for (fn, fk, fc), (cn, ck, cc) in zip(f_fields, c_fields):
        assert fk == kinds[ck] and fc == cc, (fn, fk, ck)


def test_constants_and_line_length():
    text, _ = _c_declarations()
    c_codes = {}
    for m in re.finditer(r"#define\s+(DG_\w+)\s+(\(?-?\d+(?:\s*<<\s*\d+)?\)?)", text):
        expr = m.group(2).strip("()")
        base, _, shift = expr.partition("<<")
        c_codes[m.group(1)] = int(base) << int(shift) if shift else int(base)
    assert {"DG_OK", "DG_ERR_NAN", "DG_SPLIT_PI", "DG_NOALLOC_MAX_ELEMS"} <= set(c_codes)
    f_codes = {}
    for st in _fortran_statements():
        m = re.match(r"INTEGER\(C_INT\),\s*PARAMETER\s*::\s*(DG_\w+)\s*=\s*(-?\d+)", st)
        if m:
            f_codes[m.group(1)] = int(m.group(2))
    assert f_codes == c_codes
    for i, line in enumerate(open(F90), 1):
        assert len(line.rstrip("\n")) <= 132, "line %d longer than 132 characters" % i
