"""CPU checks of the C ABI: the library loads and exports what the headers declare."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT

HEADERS = sorted(glob.glob(os.path.join(ROOT, "include", "*.h")))
DECL = re.compile(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(lulesh_\w+)\s*\(", re.M)


def declared_functions():
    names = []
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += [n for n in DECL.findall(text)]
    return sorted(set(names))


def enum_values(header, prefix):
    text = re.sub(r"/\*.*?\*/", "", open(header).read(), flags=re.S)
    vals, cur = {}, -1
    for m in re.finditer(r"\b(" + prefix + r"\w+)\s*(?:=\s*(\d+))?\s*[,}\n]", text):
        cur = int(m.group(2)) if m.group(2) else cur + 1
        vals[m.group(1)] = cur
    return vals


def test_headers_declare_functions():
    names = declared_functions()
    assert "lulesh_create" in names and "lulesh_lagrange_leapfrog" in names
    assert len(names) >= 18


def test_library_exports_every_declared_symbol(gpu_lib):
    lib = ctypes.CDLL(gpu_lib.library_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_calls_that_need_no_gpu(gpu_lib):
    L = gpu_lib.load_library()
    p = gpu_lib._Params()
    L.lulesh_default_params(ctypes.byref(p), 30)
    assert (p.nx, p.nr, p.balance, p.cost, p.mode) == (30, 11, 1, 1, 0)
    assert L.lulesh_status_string(2) == b"QStopError"
    assert L.lulesh_kernel_name(1) == b"k_force"
    # invalid problems are rejected before any CUDA call
    h = ctypes.c_void_p()
    p.nx = 0
    assert L.lulesh_create(ctypes.byref(p), ctypes.byref(h)) == 6
    p.nx, p.mode = 8, 9
    assert L.lulesh_create(ctypes.byref(p), ctypes.byref(h)) == 6
    assert L.lulesh_destroy(None) == 6
    assert L.lulesh_adj_set_overlap(None, 1) == 6


def test_python_ids_match_header(gpu_lib):
    h = os.path.join(ROOT, "include", "lulesh_gb300.h")
    fields = enum_values(h, "LULESH_F_")
    for name, (fid, _) in gpu_lib.FIELDS.items():
        key = "LULESH_F_" + name.upper()
        assert fields[key] == fid, name
    scal = enum_values(h, "LULESH_S_")
    for name, sid in gpu_lib.SCALARS.items():
        assert scal["LULESH_S_" + name.upper()] == sid, name


def test_no_fallback_without_library(tmp_path, monkeypatch):
    import lulesh_gb300
    monkeypatch.setenv("LULESH_GB300_LIB", str(tmp_path / "missing.so"))
    monkeypatch.setattr(lulesh_gb300, "_LIB", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        lulesh_gb300.load_library()


def test_struct_layouts_match_header(gpu_lib, tmp_path):
    """Every struct the Python mirror passes across the ABI has the header's
    size and field offsets (a C program built against include/ prints them)."""
    structs = {"lulesh_params": gpu_lib._Params, "lulesh_scalars": gpu_lib._Scalars,
               "lulesh_instance": gpu_lib.Instance, "lulesh_tuning": gpu_lib.Tuning,
               "lulesh_adj_result": gpu_lib.AdjResult, "lulesh_force_args": gpu_lib.ForceArgs}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "lulesh_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    import subprocess
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln:
            parts = ln.split()
            got[(parts[0], parts[1])] = int(parts[2])
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
