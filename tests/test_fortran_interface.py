"""The Fortran interface modules (include/galaexi_gb300.f90, and the CUDA Fortran module
include/galaexi_gb300_cuf.cuf) against the C header and the library.

No Fortran compiler exists in this image, so the module is checked by reading it: every function the C
header declares has exactly one BIND(C) procedure with the same number of arguments, exported by
libgalaexi_gb300.so; the BIND(C) dg_config type lists the C struct's fields in the same order with
matching kinds; every argument is passed as its C parameter expects (scalars by value, pointers
by reference to data of the same kind or as TYPE(C_PTR) values); the integer parameters equal
the header's #define constants, all of which are present; and every line fits Fortran's
132-character free-form limit.
"""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "include", "galaexi_gb300.f90")
HDR = os.path.join(ROOT, "include", "galaexi_gb300.h")


def _fortran_statements(path=F90):
    """Free-form statements with continuation lines joined and comments dropped."""
    out, cur = [], ""
    for line in open(path):
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


def _c_param(decl):
    """(base type, pointer depth) of a C parameter declaration such as 'const double* d_U'."""
    depth = decl.count("*")
    words = [w for w in re.split(r"[\s\*]+", decl) if w and w != "const"]
    return " ".join(words[:-1]), depth


def _fortran_interfaces():
    """{C name: (result kind or None, [(dummy, type spec, has VALUE)])} of the interface block."""
    out, cur = {}, None
    for st in _fortran_statements():
        m = re.match(r"(?:(.+?)\s+)?(FUNCTION|SUBROUTINE)\s+(\w+)\s*\(([^)]*)\)\s*BIND\s*\(\s*C\s*,\s*NAME\s*=\s*'(\w+)'",
                     st, flags=re.I)
        if m:
            dummies = [a.strip() for a in m.group(4).split(",") if a.strip()]
            cur = {"result": (m.group(1) or "").upper() or None, "dummies": dummies, "decl": {}}
            out[m.group(5)] = cur
            continue
        if cur is None or re.match(r"(IMPORT|END\s)", st, flags=re.I):
            if re.match(r"END\s+(FUNCTION|SUBROUTINE)", st, flags=re.I):
                cur = None
            continue
        spec, names = st.split("::")
        attrs = [a.strip().upper() for a in spec.split(",")]
        for nm in re.split(r",(?![^(]*\))", names):
            cur["decl"][re.match(r"\s*(\w+)", nm).group(1).lower()] = (attrs[0], "VALUE" in attrs[1:])
    return {k: (v["result"], [(d, *v["decl"][d.lower()]) for d in v["dummies"]]) for k, v in out.items()}


def test_bind_c_argument_passing_matches_c_types():
    """Each dummy is passed as the C parameter expects: scalars by value, pointers either by reference
    (host data of the same kind) or as a TYPE(C_PTR) value (device or opaque pointers)."""
    text, decls = _c_declarations()
    rets = {m.group(2): m.group(1).splitlines()[-1].replace("const", "").strip()
            for m in re.finditer(r"\b([A-Za-z_][\w\s\*]*?)\b(dg_\w+)\s*\([^;{}]*?\)\s*;", text)}
    kind = {"int": "INTEGER(C_INT)", "double": "REAL(C_DOUBLE)", "size_t": "INTEGER(C_SIZE_T)",
            "long long": "INTEGER(C_LONG_LONG)", "char": "CHARACTER(KIND=C_CHAR)"}
    ifaces = _fortran_interfaces()
    assert sorted(ifaces) == sorted(decls)
    for cname, (result, dummies) in ifaces.items():
        ret = rets[cname]
        if ret == "void":
            assert result is None, cname
        elif ret.replace(" ", "") == "char*":
            assert result == "TYPE(C_PTR)", cname
        else:
            assert result == kind[ret], (cname, ret, result)
        for (dname, ftype, by_value), cdecl in zip(dummies, decls[cname]):
            base, depth = _c_param(cdecl)
            what = (cname, dname, cdecl, ftype, by_value)
            if depth == 0:
                assert ftype == kind[base] and by_value, what
            elif base in ("void", "dg_ctx") and depth == 1:
                assert ftype == "TYPE(C_PTR)" and by_value, what
            elif base == "dg_ctx" and depth == 2:
                assert ftype == "TYPE(C_PTR)" and not by_value, what
            elif base == "dg_config":
                assert ftype == "TYPE(DG_CONFIG)" and not by_value, what
            else:
                assert depth == 1, what
                assert (ftype == kind[base] and not by_value) or (ftype == "TYPE(C_PTR)" and by_value), what


CUF = os.path.join(ROOT, "include", "galaexi_gb300_cuf.cuf")
INTEGRATION = os.path.join(ROOT, "INTEGRATION.md")
STREAM_KIND = "INTEGER(KIND=CUDA_STREAM_KIND)"


def _cuf_interfaces():
    """{Fortran name: (C name, [(dummy, type spec, attributes)])} of MOD_GB300_CUF."""
    out, cur = {}, None
    for st in _fortran_statements(CUF):
        m = re.match(r"(?:(.+?)\s+)?(FUNCTION|SUBROUTINE)\s+(\w+)\s*\(([^)]*)\)\s*BIND\s*\(\s*C\s*,\s*NAME\s*=\s*'(\w+)'",
                     st, flags=re.I)
        if m:
            cur = {"c": m.group(5), "dummies": [a.strip() for a in m.group(4).split(",") if a.strip()], "decl": {}}
            out[m.group(3).lower()] = cur
            continue
        if cur is None or re.match(r"(IMPORT|END\s)", st, flags=re.I):
            if re.match(r"END\s+(FUNCTION|SUBROUTINE)", st, flags=re.I):
                cur = None
            continue
        spec, names = st.split("::")
        attrs = [a.strip().upper() for a in re.split(r",(?![^(]*\))", spec)]
        for nm in re.split(r",(?![^(]*\))", names):
            cur["decl"][re.match(r"\s*(\w+)", nm).group(1).lower()] = (attrs[0], set(attrs[1:]))
    return {k: (v["c"], [(d, *v["decl"][d.lower()]) for d in v["dummies"]]) for k, v in out.items()}


def test_cuda_fortran_interfaces_match_header():
    """MOD_GB300_CUF binds every entry point that takes a stream; device-pointer parameters (d_*) are
    DEVICE arrays, the stream is a CUDA_STREAM_KIND value, the context a TYPE(C_PTR) value, host
    pointers are host data of the C parameter's kind, scalars are values."""
    _, decls = _c_declarations()
    kind = {"int": "INTEGER(C_INT)", "double": "REAL(C_DOUBLE)", "size_t": "INTEGER(C_SIZE_T)",
            "long long": "INTEGER(C_LONG_LONG)"}
    ifaces = _cuf_interfaces()
    with_stream = {c for c, args in decls.items() if args and args[-1].replace(" ", "") == "void*stream"}
    assert sorted(c for c, _ in ifaces.values()) == sorted(with_stream)
    for fname, (cname, dummies) in ifaces.items():
        assert fname == "gb300_" + cname[3:], fname
        assert len(dummies) == len(decls[cname]), cname
        for (dname, ftype, attrs), cdecl in zip(dummies, decls[cname]):
            base, depth = _c_param(cdecl)
            cvar = re.split(r"[\s\*]+", cdecl.strip())[-1]
            what = (cname, dname, cdecl, ftype, attrs)
            if cvar == "stream":
                assert ftype == STREAM_KIND and "VALUE" in attrs, what
            elif base == "dg_ctx":
                assert ftype == "TYPE(C_PTR)" and "VALUE" in attrs, what
            elif depth == 0:
                assert ftype == kind[base] and "VALUE" in attrs, what
            elif cvar.startswith("d_"):
                assert ftype == kind[base] and "DEVICE" in attrs and "VALUE" not in attrs, what
            else:
                assert ftype == kind[base] and not attrs & {"DEVICE", "VALUE"}, what
    for i, line in enumerate(open(CUF), 1):
        assert len(line.rstrip("\n")) <= 132, "line %d longer than 132 characters" % i


def test_integration_call_sites_use_the_cuda_fortran_interfaces():
    """Every gb300_* call in the integration notes names a MOD_GB300_CUF interface with its argument
    count and passes one of the reference's streams (MOD_GPU, gpu.f90:23-45)."""
    ifaces = _cuf_interfaces()
    text, calls = open(INTEGRATION).read(), []
    for m in re.finditer(r"iErr = (gb300_\w+)\(", text):
        depth, k = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(text[k], 0)
            k += 1
        calls.append((m.group(1), text[m.end():k - 1]))
    assert {c for c, _ in calls} >= {"gb300_rhs", "gb300_lserk_step", "gb300_calc_timestep"}
    streams = {"defaultstream"} | {"stream%d" % k for k in range(1, 7)}
    for fname, arglist in calls:
        args = [a.strip() for a in re.split(r",(?![^(]*\))", arglist)]
        assert fname in ifaces, fname
        assert len(args) == len(ifaces[fname][1]), (fname, args)
        assert args[-1].lower() in streams, (fname, args[-1])
        assert not any("C_DEVLOC" in a or "C_NULL_PTR" in a for a in args), (fname, args)
