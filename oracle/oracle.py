"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the parity reference or the timed CPU baseline. The oracle restates
LULESH.jl's Domain setup and LagrangeLeapFrog step (see lulesh_oracle.hpp).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")

FAITHFUL = 0
FIX_NORMALS = 1
FIX_VOLUDER = 2
FIX_LXIP = 4
LULESH2 = 7

_libs = {}


def build():
    """Compile the oracle with its Makefile (outputs in oracle/_build)."""
    r = subprocess.run(["make", "-s", "-C", HERE, "-j4"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def load(openmp=True):
    key = "omp" if openmp else "serial"
    if key in _libs:
        return _libs[key]
    path = os.path.join(BUILD, "liblulesh_oracle_omp.so" if openmp else "liblulesh_oracle.so")
    if not os.path.exists(path):
        build()
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    L.ora_create.restype = P
    L.ora_create.argtypes = [ctypes.c_int] * 5 + [ctypes.c_ulonglong]
    for f in ["ora_destroy"]:
        getattr(L, f).argtypes = [P]
        getattr(L, f).restype = None
    for f in ["ora_time_increment", "ora_lagrange_leapfrog", "ora_lagrange_nodal",
              "ora_lagrange_elements", "ora_force_for_nodes", "ora_time_constraints",
              "ora_error_site"]:
        getattr(L, f).argtypes = [P]
        getattr(L, f).restype = ctypes.c_int
    for f in ["ora_num_elem", "ora_num_node", "ora_cycle", "ora_error_index"]:
        getattr(L, f).argtypes = [P]
        getattr(L, f).restype = ctypes.c_longlong
    L.ora_set_cycle.argtypes = [P, ctypes.c_longlong]
    L.ora_run.argtypes = [P, ctypes.c_longlong]
    L.ora_run.restype = ctypes.c_int
    L.ora_field_f64.argtypes = [P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_longlong)]
    L.ora_field_f64.restype = ctypes.POINTER(ctypes.c_double)
    L.ora_field_i64.argtypes = [P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_longlong)]
    L.ora_field_i64.restype = ctypes.POINTER(ctypes.c_longlong)
    L.ora_elem_bc.argtypes = [P, ctypes.POINTER(ctypes.c_longlong)]
    L.ora_elem_bc.restype = ctypes.POINTER(ctypes.c_uint)
    L.ora_get_scalar.argtypes = [P, ctypes.c_char_p, ctypes.POINTER(ctypes.c_double)]
    L.ora_set_scalar.argtypes = [P, ctypes.c_char_p, ctypes.c_double]
    L.ora_symmetry.argtypes = [P, ctypes.POINTER(ctypes.c_double)]
    L.ora_set_einit.argtypes = [P, ctypes.c_double]
    L.ora_set_einit.restype = None
    L.ora_max_threads.restype = ctypes.c_int
    L.ora_set_threads.argtypes = [ctypes.c_int]
    _libs[key] = L
    return L


I64_FIELDS = {"matElemlist", "nodelist", "lxim", "lxip", "letam", "letap", "lzetam", "lzetap",
              "symmX", "symmY", "symmZ", "nodeElemCount", "nodeElemStart", "nodeElemCornerList",
              "regElemSize", "regCSR", "regReps", "regNumList", "regElemlist", "regSorted"}


class OracleDomain:
    """One oracle problem; fields are numpy views of the oracle's storage."""

    def __init__(self, nx, nr=11, balance=1, cost=1, mode=FAITHFUL, seed=0, openmp=True, threads=0):
        self.L = load(openmp)
        if threads:
            self.L.ora_set_threads(int(threads))
        self.h = self.L.ora_create(int(nx), int(nr), int(balance), int(cost), int(mode), int(seed))
        if not self.h:
            raise ValueError("bad oracle parameters")
        self.nx = nx

    def close(self):
        if self.h:
            self.L.ora_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def view(self, name):
        n = ctypes.c_longlong()
        if name == "elemBC":
            p = self.L.ora_elem_bc(self.h, ctypes.byref(n))
            return np.ctypeslib.as_array(p, (n.value,))
        if name in I64_FIELDS:
            p = self.L.ora_field_i64(self.h, name.encode(), ctypes.byref(n))
        else:
            p = self.L.ora_field_f64(self.h, name.encode(), ctypes.byref(n))
        if not p:
            raise KeyError(name)
        return np.ctypeslib.as_array(p, (n.value,))

    def field(self, name):
        return self.view(name).copy()

    def set_field(self, name, values):
        v = self.view(name)
        v[:] = values

    def get(self, name):
        if name == "cycle":
            return int(self.L.ora_cycle(self.h))
        x = ctypes.c_double()
        if self.L.ora_get_scalar(self.h, name.encode(), ctypes.byref(x)) != 0:
            raise KeyError(name)
        return x.value

    def set(self, name, value):
        if name == "cycle":
            self.L.ora_set_cycle(self.h, int(value))
            return
        if self.L.ora_set_scalar(self.h, name.encode(), float(value)) != 0:
            raise KeyError(name)

    def set_einit(self, einit):
        """Deposit `einit` in the origin element (and recompute the initial dt)."""
        self.L.ora_set_einit(self.h, float(einit))

    def time_increment(self):
        self.L.ora_time_increment(self.h)

    def lagrange_leapfrog(self):
        return self.L.ora_lagrange_leapfrog(self.h)

    def lagrange_nodal(self):
        return self.L.ora_lagrange_nodal(self.h)

    def lagrange_elements(self):
        return self.L.ora_lagrange_elements(self.h)

    def time_constraints(self):
        return self.L.ora_time_constraints(self.h)

    def run(self, num_iters):
        return self.L.ora_run(self.h, int(num_iters))

    def error_site(self):
        return self.L.ora_error_site(self.h)

    def symmetry(self):
        out = (ctypes.c_double * 3)()
        self.L.ora_symmetry(self.h, out)
        return tuple(out)


def load_dual():
    """The dual-number (forward-mode) build of the oracle."""
    if "dual" in _libs:
        return _libs["dual"]
    path = os.path.join(BUILD, "liblulesh_oracle_dual.so")
    if not os.path.exists(path):
        build()
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    D = ctypes.POINTER(ctypes.c_double)
    L.ord_create.restype = P
    L.ord_create.argtypes = [ctypes.c_int] * 5 + [ctypes.c_ulonglong]
    L.ord_destroy.argtypes = [P]
    L.ord_destroy.restype = None
    for f in ["ord_num_elem", "ord_num_node", "ord_cycle"]:
        getattr(L, f).argtypes = [P]
        getattr(L, f).restype = ctypes.c_longlong
    L.ord_set_cycle.argtypes = [P, ctypes.c_longlong]
    L.ord_set_cycle.restype = None
    L.ord_set_field.argtypes = [P, ctypes.c_char_p, D, D, ctypes.c_longlong]
    L.ord_get_field.argtypes = [P, ctypes.c_char_p, D, D, ctypes.c_longlong]
    L.ord_set_scalar.argtypes = [P, ctypes.c_char_p, ctypes.c_double, ctypes.c_double]
    L.ord_get_scalar.argtypes = [P, ctypes.c_char_p, D, D]
    for f in ["ord_time_increment", "ord_lagrange_leapfrog"]:
        getattr(L, f).argtypes = [P]
        getattr(L, f).restype = ctypes.c_int
    L.ord_cycles.argtypes = [P, ctypes.c_longlong]
    L.ord_cycles.restype = ctypes.c_int
    _libs["dual"] = L
    return L


def _dptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class DualDomain:
    """An oracle problem over dual numbers: every value carries one tangent,
    so running cycles gives the exact Jacobian-vector product of the run."""

    def __init__(self, nx, nr=11, balance=1, cost=1, mode=FAITHFUL, seed=0):
        self.L = load_dual()
        self.h = self.L.ord_create(int(nx), int(nr), int(balance), int(cost), int(mode), int(seed))
        if not self.h:
            raise ValueError("bad oracle parameters")
        self.ne = int(self.L.ord_num_elem(self.h))
        self.nn = int(self.L.ord_num_node(self.h))

    def close(self):
        if self.h:
            self.L.ord_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _len(self, name):
        node = name in ("x", "y", "z", "xd", "yd", "zd", "xdd", "ydd", "zdd", "fx", "fy", "fz", "nodalMass")
        return self.nn if node else self.ne

    def set_field(self, name, values=None, tangents=None):
        n = self._len(name)
        v = None if values is None else np.ascontiguousarray(values, dtype=np.float64)
        t = None if tangents is None else np.ascontiguousarray(tangents, dtype=np.float64)
        if self.L.ord_set_field(self.h, name.encode(), _dptr(v), _dptr(t), n) != 0:
            raise KeyError(name)

    def field(self, name):
        """(values, tangents) of a field."""
        n = self._len(name)
        v = np.empty(n)
        t = np.empty(n)
        if self.L.ord_get_field(self.h, name.encode(), _dptr(v), _dptr(t), n) != 0:
            raise KeyError(name)
        return v, t

    def get(self, name):
        if name == "cycle":
            return int(self.L.ord_cycle(self.h)), 0.0
        v, t = ctypes.c_double(), ctypes.c_double()
        if self.L.ord_get_scalar(self.h, name.encode(), ctypes.byref(v), ctypes.byref(t)) != 0:
            raise KeyError(name)
        return v.value, t.value

    def set(self, name, value, tangent=0.0):
        if name == "cycle":
            self.L.ord_set_cycle(self.h, int(value))
            return
        if self.L.ord_set_scalar(self.h, name.encode(), float(value), float(tangent)) != 0:
            raise KeyError(name)

    def cycles(self, n):
        return self.L.ord_cycles(self.h, int(n))
