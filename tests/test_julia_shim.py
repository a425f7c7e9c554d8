"""The Julia binding (``treeamr.jl_gb300/julia/TreeAMRCUDA.jl``) against the
C ABI it calls (``include/treeamr_cuda.h``), read as text: there is no Julia
toolchain to run it.  Every struct the shim mirrors has the header's fields in
the header's order and widths; every ``ccall`` names a declared function with
its number of arguments, each a pointer where the header has one and a scalar
of the header's width where it has a scalar; the option codes are the
header's, in the shim and in the Python host's tables."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "treeamr_cuda.h")
SHIM = os.path.join(ROOT, "treeamr.jl_gb300", "julia", "TreeAMRCUDA.jl")

STRUCTS = {"tam_stencil": "TamStencil", "tam_group": "TamGroup",
           "tam_schedule_desc": "TamScheduleDesc", "tam_state_layout": "TamStateLayout"}
SCALARS = {"int32_t": "Int32", "int64_t": "Int64", "uint64_t": "UInt64", "int": "Int32",
           "double": "Float64", "size_t": "UInt64"}
JULIA_ALIASES = {"Cint": "Int32", "Csize_t": "UInt64", "Cdouble": "Float64",
                 "Clong": "Int64", "UInt8": "UInt8"}


def _header():
    text = open(HEADER).read()
    return re.sub(r"/\*.*?\*/", "", text, flags=re.S)


def _shim():
    return "\n".join(line.split("#", 1)[0] for line in open(SHIM).read().splitlines())


def _c_fields(text, name):
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), text, flags=re.S)
    assert m, name
    out = []
    for decl in m.group(1).split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        arr = re.match(r"(.*?)(\w+)\[(\w+)\]$", decl)
        if arr:
            ctype, field, n = arr.group(1).strip(), arr.group(2), arr.group(3)
            n = 3 if n == "TAM_MAX_DIM" else int(n)
            out.append((field, "NTuple{%d,%s}" % (n, _c_to_julia(ctype))))
            continue
        ptr = re.match(r"(?:const )?(\w+) \*(\w+)$", decl)
        if ptr:
            out.append((ptr.group(2), "Ptr{%s}" % _c_to_julia(ptr.group(1), pointee=True)))
            continue
        ctype, field = decl.rsplit(" ", 1)
        out.append((field, _c_to_julia(ctype)))
    return out


def _c_to_julia(ctype, pointee=False):
    ctype = ctype.replace("const ", "").strip()
    if ctype in STRUCTS:
        return STRUCTS[ctype]
    if ctype == "void" and pointee:
        return "Cvoid"
    return SCALARS[ctype]


def _julia_fields(text, name):
    m = re.search(r"\nstruct %s\n(.*?)\nend" % name, text, flags=re.S)
    assert m, name
    out = []
    for line in m.group(1).splitlines():
        line = line.strip()
        if not line:
            continue
        field, jtype = line.split("::", 1)
        jtype = jtype.strip()
        for k, v in JULIA_ALIASES.items():
            jtype = re.sub(r"\b%s\b" % k, v, jtype)
        out.append((field.strip(), jtype))
    return out


def _c_functions(text):
    out = {}
    for m in re.finditer(r"\b(?:int|void)\s+(tam_\w+)\s*\(([^;{]*?)\)\s*;", text, flags=re.S):
        params = [" ".join(p.split()) for p in m.group(2).split(",")]
        out[m.group(1)] = [] if params == ["void"] else params
    return out


def _split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch in "({":
            depth += 1
        elif ch in ")}":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur.strip())
            cur = ""
        else:
            cur += ch
    if cur.strip():
        parts.append(cur.strip())
    return [p for p in parts if p]


def _ccalls(text):
    out = []
    for m in re.finditer(r"ccall\(\(:(\w+), LIB\),\s*(\w+),\s*\(", text):
        i, depth = m.end(), 1
        j = i
        while depth:
            depth += {"(": 1, ")": -1}.get(text[j], 0)
            j += 1
        out.append((m.group(1), _split_top(text[i:j - 1])))
    return out


def _kind_c(param):
    if "*" in param:
        return "ptr"
    ctype = param.replace("const ", "").rsplit(" ", 1)[0]
    return SCALARS[ctype]


def _kind_julia(jtype):
    if re.match(r"(Ptr|CuPtr|Ref)\{", jtype):
        return "ptr"
    return JULIA_ALIASES.get(jtype, jtype)


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_structs_match_the_header(cname):
    c = _c_fields(_header(), cname)
    j = _julia_fields(_shim(), STRUCTS[cname])
    assert j == c, (cname, c, j)


def test_a_changed_field_is_caught():
    """The comparison is not vacuous: a shim whose layout struct had a
    32-bit block count, or lost a field, no longer matches."""
    c = _c_fields(_header(), "tam_state_layout")
    text = _shim()
    wide = text.replace("    nblocks::Int64\nend", "    nblocks::Int32\nend", 1)
    assert wide != text
    assert _julia_fields(wide, "TamStateLayout") != c
    short = text.replace("    nvars::Int32\n    nblocks::Int64\nend", "    nblocks::Int64\nend", 1)
    assert short != text
    assert _julia_fields(short, "TamStateLayout") != c


def test_every_ccall_matches_its_declaration():
    funcs = _c_functions(_header())
    calls = _ccalls(_shim())
    assert len(calls) >= 10
    for name, jargs in calls:
        assert name in funcs, name
        cargs = funcs[name]
        assert len(jargs) == len(cargs), (name, cargs, jargs)
        for cp, jt in zip(cargs, jargs):
            assert _kind_c(cp) == _kind_julia(jt), (name, cp, jt)


def test_dynamic_fill_calls_match_tam_fill():
    """``tam_fill!`` calls tam_fill or tam_fill_plain through one ccall whose
    name is a variable; both take the same arguments."""
    funcs = _c_functions(_header())
    assert funcs["tam_fill"] == funcs["tam_fill_plain"]
    m = re.search(r"ccall\(\(f, LIB\), Cint,\s*\((.*?)\),\s*ds\.handle", _shim(), flags=re.S)
    assert m
    jargs = _split_top(m.group(1))
    assert [_kind_julia(t) for t in jargs] == [_kind_c(p) for p in funcs["tam_fill"]]


def test_option_codes_match_the_header():
    defines = {k.lower(): int(v) for k, v in
               re.findall(r"#define TAM_OPT_(\w+) (\d+)", _header())}
    m = re.search(r"const OPTIONS = \((.*?)\)\n", _shim(), flags=re.S)
    assert m
    shim = {k: int(v) for k, v in re.findall(r"(\w+)=Int32\((\d+)\)", m.group(1))}
    assert shim == defines


def test_abi_version_matches():
    v = int(re.search(r"#define TAM_ABI_VERSION (\d+)", _header()).group(1))
    assert re.search(r"const TAM_ABI_VERSION = Int32\(%d\)" % v, _shim())


def test_python_option_codes_match_the_header():
    """The Python host's option tables (one schedule's and a batch's, the
    batch taking a subset) carry the header's codes."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "treeamr.jl_gb300"))
    from treeamr.batch import ForestBatch
    from treeamr.ghosts import DeviceSchedule
    defines = {k.lower(): int(v) for k, v in
               re.findall(r"#define TAM_OPT_(\w+) (\d+)", _header())}
    assert DeviceSchedule.OPTIONS == defines
    assert ForestBatch.OPTIONS.items() <= defines.items()
    assert set(defines) - set(ForestBatch.OPTIONS) == {"block_order", "merge_stages"}
