"""The Fortran interface module (include/mdt_gpu.f90) covers the C header
(include/mdt_gpu.h): every function has a bind(C) interface with the same symbol, the
same number of arguments and compatible C kinds, every struct a bind(C) type with the same
fields in the same order and kinds, and every status / id macro a parameter of the same
value.  No Fortran compiler exists on either build machine, so this is the check that
keeps the two files from drifting apart."""
import re
from pathlib import Path

INC = Path(__file__).resolve().parent.parent / "include"

C_SCALAR = {"int32_t": "c_int32_t", "int64_t": "c_int64_t", "uint64_t": "c_int64_t", "double": "c_double",
            "uint8_t": "c_int8_t", "char": "c_char", "void": "void"}


def _strip_c(text):
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def _c_decl(decl):
    """'const double *x' -> ('x', base kind, pointer depth)."""
    decl = decl.replace("const ", " ").strip()
    m = re.match(r"([A-Za-z_][A-Za-z0-9_]*)\s*(\**)\s*([A-Za-z_][A-Za-z0-9_]*)$", decl)
    assert m, decl
    base, stars, name = m.groups()
    return name, C_SCALAR.get(base, base), len(stars)


def parse_header():
    text = _strip_c((INC / "mdt_gpu.h").read_text())
    structs = {}
    for body, name in re.findall(r"typedef struct \w+ \{(.*?)\}\s*(\w+);", text, flags=re.S):
        fields = []
        for stmt in body.split(";"):
            stmt = stmt.replace("const ", " ").strip()
            if not stmt:
                continue
            base, rest = stmt.split(None, 1)
            for d in rest.split(","):
                d = d.strip()
                stars = len(d) - len(d.lstrip("*"))
                fields.append((d.lstrip("*").strip(), "ptr" if stars else C_SCALAR[base]))
        structs[name] = fields
    funcs = {}
    for ret, name, args in re.findall(r"\b(int32_t|int64_t|const char \*)\s*(mdt_\w+)\s*\(([^)]*)\)\s*;", text):
        parsed = [_c_decl(a) for a in args.split(",")] if args.strip() else []
        funcs[name] = (C_SCALAR.get(ret, "ptr") if "*" not in ret else "ptr", parsed)
    macros = {k: int(v) for k, v in re.findall(r"#define\s+(MDT_\w+)\s+(-?\d+)", text)}
    return structs, funcs, macros


def _f_kind(spec):
    spec = spec.strip().lower()
    m = re.match(r"(integer|real)\((c_\w+)\)", spec)
    if m:
        return m.group(2)
    m = re.match(r"type\((\w+)\)", spec)
    assert m, spec
    return "ptr" if m.group(1) == "c_ptr" else m.group(1)


def parse_fortran():
    src = (INC / "mdt_gpu.f90").read_text()
    lines = []
    for raw in src.splitlines():
        line = raw.split("!")[0].rstrip()
        if lines and lines[-1].endswith("&"):
            lines[-1] = lines[-1][:-1] + " " + line.strip()
        else:
            lines.append(line)
    consts, types, funcs = {}, {}, {}
    cur_type = cur_fn = None
    for line in lines:
        s = line.strip()
        low = s.lower()
        for name, val in re.findall(r"(MDT_\w+)\s*=\s*(-?\d+)", s):
            consts[name] = int(val)
        m = re.match(r"type,\s*bind\(c\)\s*::\s*(\w+)", low)
        if m:
            cur_type = m.group(1)
            types[cur_type] = []
            continue
        if low.startswith("end type"):
            cur_type = None
            continue
        m = re.match(r"(.*?)\s*function\s+(\w+)\s*\(([^)]*)\)\s*bind\(c,\s*name=\"(\w+)\"\)", s, flags=re.I)
        if m:
            ret, _, args, cname = m.groups()
            cur_fn = cname
            funcs[cname] = {"ret": _f_kind(ret), "args": [a.strip().lower() for a in args.split(",") if a.strip()],
                            "decl": {}}
            continue
        if low.startswith("end function"):
            cur_fn = None
            continue
        if "::" in s and (cur_type or cur_fn) and not low.startswith("import"):
            spec, names = s.split("::", 1)
            parts = [p.strip() for p in re.split(r",(?![^(]*\))", spec)]
            kind = _f_kind(parts[0])
            value = any(p.lower() == "value" for p in parts[1:])
            for n in re.split(r",(?![^(]*\))", names):
                n = n.strip()
                nm = re.match(r"(\w+)", n).group(1).lower()
                if cur_type:
                    types[cur_type].append((nm, kind))
                else:
                    funcs[cur_fn]["decl"][nm] = (kind, value, "(" in n)
    return consts, types, funcs


def _compatible(c_arg, f_arg):
    _, ckind, depth = c_arg
    fkind, value, _ = f_arg
    if depth == 0:
        return value and fkind == ckind
    if ckind in ("mdt_ctx", "void") and depth == 1:
        return value and fkind == "ptr"
    if depth == 2:
        return not value and fkind == "ptr"
    # pointer to data: by reference with the same kind, or an explicit c_ptr by value
    return (not value and fkind == ckind) or (value and fkind == "ptr")


def test_every_header_function_has_a_matching_interface():
    _, cfuncs, _ = parse_header()
    _, _, ffuncs = parse_fortran()
    assert len(cfuncs) >= 35
    missing = sorted(set(cfuncs) - set(ffuncs))
    assert not missing, f"no bind(C) interface for {missing}"
    for name, (cret, cargs) in cfuncs.items():
        f = ffuncs[name]
        assert f["ret"] == cret, (name, f["ret"], cret)
        assert len(f["args"]) == len(cargs), (name, f["args"], cargs)
        for ca, fa_name in zip(cargs, f["args"]):
            assert fa_name in f["decl"], (name, fa_name)
            assert _compatible(ca, f["decl"][fa_name]), (name, ca, f["decl"][fa_name])


def test_every_header_struct_has_a_matching_type():
    cstructs, _, _ = parse_header()
    _, ftypes, _ = parse_fortran()
    assert set(cstructs) == set(ftypes), (sorted(cstructs), sorted(ftypes))
    for name, cfields in cstructs.items():
        ff = ftypes[name]
        assert [k for _, k in ff] == [k for _, k in cfields], (name, ff, cfields)
        assert [n for n, _ in ff] == [n.lower() for n, _ in cfields], name


def test_every_header_constant_has_a_parameter():
    _, _, macros = parse_header()
    consts, _, _ = parse_fortran()
    for k, v in macros.items():
        assert consts.get(k) == v, (k, v, consts.get(k))
