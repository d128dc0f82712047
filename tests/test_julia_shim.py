"""CPU checks of the Julia shim (julia/LULESHGB300.jl) without Julia.

Julia lays out an isbits struct like the C struct with the same fields, so a
`ccall` passes the right bytes exactly when the shim's structs have the
header's field names, order and types. The shim's structs are parsed here and
their C layout (natural alignment) is compared with the ctypes mirrors, which
tests/test_abi.py compares with the compiled header. The field and scalar ids
and the methods examples/benchmark.jl:22-110 needs are checked the same way,
and every `ccall` of the shim and of the ChainRules rule against the C
prototype it binds (return type, argument count and types).
"""
import ctypes
import os
import re

import pytest

from conftest import ROOT

SHIM = os.path.join(ROOT, "lulesh.jl_gb300", "julia", "LULESHGB300.jl")
HEADER = os.path.join(ROOT, "include", "lulesh_gb300.h")

# size = alignment of the Julia types the shim's structs use
JULIA_SIZE = {"Int32": 4, "UInt32": 4, "Int64": 8, "UInt64": 8, "Float64": 8, "Float32": 4}
CTYPE_OF = {"Int32": ctypes.c_int32, "UInt32": ctypes.c_uint32, "Int64": ctypes.c_int64,
            "UInt64": ctypes.c_uint64, "Float64": ctypes.c_double, "Float32": ctypes.c_float}


def shim_text():
    return open(SHIM).read()


def julia_structs(text):
    """{name: [(field, type), ...]} of the immutable structs whose fields are all plain types."""
    out = {}
    for m in re.finditer(r"^struct (\w+)\s*\n(.*?)^end", text, re.S | re.M):
        fields = []
        for ln in m.group(2).splitlines():
            ln = ln.split("#")[0].strip()
            if not ln:
                continue
            f = re.match(r"(\w+)::(\w+)$", ln)
            if f:
                fields.append((f.group(1), f.group(2)))
        if fields and all(t in JULIA_SIZE for _, t in fields):
            out[m.group(1)] = fields
    return out


def c_layout(fields):
    """Offsets and size of a C struct with these fields (natural alignment)."""
    off, offs, align = 0, [], 1
    for _, t in fields:
        s = JULIA_SIZE[t]
        off = (off + s - 1) // s * s
        offs.append(off)
        off += s
        align = max(align, s)
    return offs, (off + align - 1) // align * align


@pytest.mark.parametrize("jname,pyname", [("Params", "_Params"), ("Scalars", "_Scalars"),
                                          ("AdjResult", "AdjResult")])
def test_shim_structs_match_the_header(gpu_lib, jname, pyname):
    fields = julia_structs(shim_text())[jname]
    py = getattr(gpu_lib, pyname)
    assert [f for f, _ in fields] == [f for f, _ in py._fields_], jname
    for (f, t), (pf, pt) in zip(fields, py._fields_):
        assert ctypes.sizeof(CTYPE_OF[t]) == ctypes.sizeof(pt), (jname, f, t, pt)
    offs, size = c_layout(fields)
    assert size == ctypes.sizeof(py), jname
    assert offs == [getattr(py, f).offset for f, _ in fields], jname


def _julia_symbols(block):
    return re.findall(r":(\w+)", block)


def test_shim_field_and_scalar_ids_match_the_header(gpu_lib):
    from test_abi import enum_values
    text = shim_text()
    fids = enum_values(HEADER, "LULESH_F_")
    groups = {}
    for name in ("elem", "node", "idx"):
        m = re.search(name + r" = \((.*?)\)", text, re.S)
        groups[name] = _julia_symbols(m.group(1))
    base = {"elem": 0, "node": 32, "idx": 64}
    for name, syms in groups.items():
        for i, s in enumerate(syms):
            assert fids["LULESH_F_" + s.upper()] == base[name] + i, s
    assert fids["LULESH_F_ELEMBC"] == int(re.search(r"FIELD_IDS\[:elemBC\] = \(Int32\((\d+)\)", text).group(1))
    sids = enum_values(HEADER, "LULESH_S_")
    m = re.search(r"const SCALAR_IDS = .*?enumerate\(\((.*?)\)\)\)", text, re.S)
    for i, s in enumerate(_julia_symbols(m.group(1))):
        assert sids["LULESH_S_" + s.upper()] == i, s


def test_shim_error_messages_cover_every_status(gpu_lib):
    text = shim_text()
    keys = {(int(a), int(b)) for a, b in re.findall(r"\((\d), (\d)\) =>", text)}
    sites = enum_values_sites()
    for site in range(1, max(sites.values()) + 1):
        assert (1, site) in keys, site
    assert (2, 0) in keys and (3, 0) in keys


def enum_values_sites():
    from test_abi import enum_values
    return {k: v for k, v in enum_values(HEADER, "LULESH_SITE_").items() if v > 0}


# What examples/benchmark.jl:22-110 calls on and reads from its domain with
# enzyme = false: the one-rank boundary exchange (:57-64), the loop (:82-98)
# and the final report (:104).
BENCHMARK_METHODS = ["commRecv", "commSend", "commSBN", "timeIncrement!", "lagrangeLeapFrog",
                     "verifyAndWriteFinalOutput"]
BENCHMARK_PROPERTIES = ["sizeX", "sizeY", "sizeZ", "nodalMass", "stoptime", "time", "cycle", "deltatime",
                        "numElem", "e"]


def test_shim_serves_the_benchmark_script():
    text = shim_text()
    for m in BENCHMARK_METHODS:
        assert re.search(r"^(function )?LULESH\." + re.escape(m) + r"\((::)?\w*::GPUDomain|"
                         r"^(function )?LULESH\." + re.escape(m) + r"\(\w+, \w+::GPUDomain",
                         text, re.M), m
    fields = set()
    for name in ("elem", "node", "idx"):
        fields |= set(_julia_symbols(re.search(name + r" = \((.*?)\)", text, re.S).group(1)))
    scalars = set(_julia_symbols(re.search(r"const SCALAR_IDS = .*?enumerate\(\((.*?)\)\)\)", text,
                                           re.S).group(1)))
    served = fields | scalars | {"numElem", "numNode", "sizeX", "sizeY", "sizeZ"}
    for p in BENCHMARK_PROPERTIES:
        assert p in served, p
    assert re.search(r"s in \(:sizeX, :sizeY, :sizeZ\)", text)


# ---- every ccall against the header's prototype ---------------------------
CHAINRULES = os.path.join(ROOT, "lulesh.jl_gb300", "julia", "LULESHGB300ChainRules.jl")

# C parameter type -> the Julia types a ccall may declare for it
C_TO_JULIA = {
    "int32_t": {"Int32", "Cint"}, "int": {"Cint", "Int32"}, "int64_t": {"Int64"}, "double": {"Float64"},
    "uint64_t": {"UInt64"}, "double*": {"Ptr{Float64}"}, "const double*": {"Ptr{Float64}"},
    "int64_t*": {"Ptr{Int64}"}, "int32_t*": {"Ptr{Int32}"}, "const char*": {"Cstring"},
    "void*": {"Ptr{Cvoid}"}, "const void*": {"Ptr{Cvoid}"},
    "const lulesh_params*": {"Ptr{Params}"}, "lulesh_params*": {"Ptr{Params}"},
    "lulesh_scalars*": {"Ptr{Scalars}"}, "lulesh_adj_result*": {"Ptr{AdjResult}"},
}
HANDLES = ("lulesh_domain", "lulesh_adjoint", "lulesh_ensemble")


def c_prototypes():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"^\s*(int|void|const char\*)\s+(lulesh_\w+)\s*\(([^)]*)\)\s*;", text, re.M):
        args = [a.strip() for a in m.group(3).split(",") if a.strip() and a.strip() != "void"]
        types = []
        for a in args:
            a = re.sub(r"\s+\w+(\[\d*\])?$", lambda k: "*" if k.group(1) is not None else "", a)  # drop the name
            types.append(re.sub(r"\s*\*", "*", a).strip())
        out[m.group(2)] = (m.group(1), types)
    return out


def julia_ccalls(text):
    calls = []
    for m in re.finditer(r"ccall\(\(:(lulesh_\w+),\s*[\w.]+\),\s*(\w+),\s*\(", text):
        depth, i = 1, m.end()
        while depth:
            depth += {"(": 1, ")": -1}.get(text[i], 0)
            i += 1
        tup = text[m.end():i - 1]
        parts, depth, cur = [], 0, ""
        for ch in tup:
            if ch == "," and depth == 0:
                parts.append(cur.strip())
                cur = ""
                continue
            depth += {"{": 1, "}": -1}.get(ch, 0)
            cur += ch
        if cur.strip():
            parts.append(cur.strip())
        calls.append((m.group(1), m.group(2), parts))
    return calls


def compatible(ctype, jtype):
    base = ctype.replace("const ", "")
    if base.rstrip("*") in HANDLES:
        return jtype == ("Ptr{Ptr{Cvoid}}" if base.endswith("**") else "Ptr{Cvoid}")
    return jtype in C_TO_JULIA.get(ctype, set())


@pytest.mark.parametrize("path", [SHIM, CHAINRULES])
def test_every_ccall_matches_its_c_prototype(path):
    protos = c_prototypes()
    calls = julia_ccalls(open(path).read())
    assert calls, path
    for name, ret, args in calls:
        assert name in protos, name
        cret, ctypes_ = protos[name]
        assert (ret in ("Cint", "Int32")) if cret == "int" else (ret == "Cvoid") if cret == "void" else True, name
        assert len(args) == len(ctypes_), (name, args, ctypes_)
        for c, j in zip(ctypes_, args):
            assert compatible(c, j), (name, c, j)
