"""Python mirror of LULESH.jl's single-rank API over liblulesh_gb300.so.

The reference's public surface (src/LULESH.jl:58-60) is `LuleshProblem`,
`Domain`, `timeIncrement!`, `lagrangeLeapFrog` and
`verifyAndWriteFinalOutput`; this module keeps those names and their meaning
(`timeIncrement!` is spelled `timeIncrement`). The state lives on the GPU;
`Domain` attributes read or write it through the C ABI declared in
include/lulesh_gb300.h. Errors the reference raises with `error(...)` raise
`LuleshError` with the same message.

There is no CPU fallback: importing works without a GPU, but creating a
Domain needs the compiled library and a CUDA device, and fails loudly
otherwise.
"""
import ctypes
import os

import numpy as np

__all__ = [
    "LuleshProblem", "Domain", "timeIncrement", "lagrangeLeapFrog", "run",
    "verifyAndWriteFinalOutput", "LuleshError", "load_library", "library_path",
    "FIELDS", "SCALARS", "MODE_FAITHFUL", "MODE_LULESH2", "Ensemble", "sedov_instances",
    "Adjoint", "STATE_FIELDS", "partition", "shard", "read_state", "block_plan",
]

_HERE = os.path.dirname(os.path.abspath(__file__))
_PKG = os.path.dirname(_HERE)

MODE_FAITHFUL = 0
FIX_NORMALS = 1
FIX_VOLUDER = 2
FIX_LXIP = 4
MODE_LULESH2 = 7

# lulesh_field ids (include/lulesh_gb300.h) -> (id, kind)
_ELEM_F64 = ["e", "p", "q", "ql", "qq", "v", "volo", "delv", "vdov", "arealg", "ss", "elemMass",
             "vnew", "delv_xi", "delv_eta", "delv_zeta", "delx_xi", "delx_eta", "delx_zeta",
             "dxx", "dyy", "dzz"]
_NODE_F64 = ["x", "y", "z", "xd", "yd", "zd", "xdd", "ydd", "zdd", "fx", "fy", "fz", "nodalMass"]
_I64 = ["nodelist", "lxim", "lxip", "letam", "letap", "lzetam", "lzetap", "symmX", "symmY",
        "symmZ", "nodeElemCount", "nodeElemStart", "nodeElemCornerList", "matElemlist",
        "regNumList", "regElemlist", "regCSR", "regReps", "regSorted", "regElemSize"]
FIELDS = {}
for _i, _n in enumerate(_ELEM_F64):
    FIELDS[_n] = (_i, np.float64)
for _i, _n in enumerate(_NODE_F64):
    FIELDS[_n] = (32 + _i, np.float64)
for _i, _n in enumerate(_I64):
    FIELDS[_n] = (64 + _i, np.int64)
FIELDS["elemBC"] = (96, np.uint32)

SCALARS = {n: i for i, n in enumerate([
    "dtfixed", "deltatimemultlb", "deltatimemultub", "stoptime", "dtmax", "dthydro", "dtcourant",
    "time", "deltatime", "u_cut", "hgcoef", "qstop", "monoq_max_slope", "monoq_limiter_mult",
    "e_cut", "p_cut", "ss4o3", "q_cut", "v_cut", "qlc_monoq", "qqc_monoq", "qqc", "eosvmax",
    "eosvmin", "pmin", "emin", "dvovmax", "refdens", "cycle"])}

# Reference messages per (status, site): src/domain.jl error(...) calls.
_MESSAGES = {
    (1, 1): "Early Volume Error",
    (1, 2): "Volume Error: Volume is negative",
    (1, 3): "Mid Volume Error",
    (1, 4): "Volume Error: calcKinematicsForElems",
    (1, 5): "Volume Error :2157",
    (1, 6): "Volume Error :2887",
    (1, 7): "Volume Error :2908",
    (2, 0): "QStopError",
    (3, 0): "Error",
}


class LuleshError(RuntimeError):
    """A step error; `.status` and `.site` hold the C ABI codes."""

    def __init__(self, msg, status=0, site=0):
        super().__init__(msg)
        self.status = status
        self.site = site


class _Params(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int32), ("nr", ctypes.c_int32), ("balance", ctypes.c_int32),
                ("cost", ctypes.c_int32), ("mode", ctypes.c_int32), ("region_reps", ctypes.c_int32),
                ("keep_aux", ctypes.c_int32), ("device", ctypes.c_int32),
                ("region_seed", ctypes.c_uint64)]


class _Scalars(ctypes.Structure):
    _fields_ = [("time", ctypes.c_double), ("deltatime", ctypes.c_double),
                ("dtcourant", ctypes.c_double), ("dthydro", ctypes.c_double),
                ("cycle", ctypes.c_int64), ("status", ctypes.c_int32), ("site", ctypes.c_int32)]


class Instance(ctypes.Structure):
    """lulesh_instance: one Sedov problem of an ensemble."""
    _fields_ = [("nx", ctypes.c_int32), ("nr", ctypes.c_int32), ("balance", ctypes.c_int32),
                ("cost", ctypes.c_int32), ("einit", ctypes.c_double), ("hgcoef", ctypes.c_double),
                ("region_seed", ctypes.c_uint64)]


class Tuning(ctypes.Structure):
    """lulesh_tuning: threads per block of the four step kernels and the
    geometry split (0 stored by k_kinematics, 1 formed in k_force)."""
    _fields_ = [("force_block", ctypes.c_int32), ("node_block", ctypes.c_int32),
                ("kin_block", ctypes.c_int32), ("mat_block", ctypes.c_int32),
                ("geometry", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AdjResult(ctypes.Structure):
    """lulesh_adj_result."""
    _fields_ = [("loss", ctypes.c_double), ("grad_hgcoef", ctypes.c_double),
                ("forward_ms", ctypes.c_double), ("reverse_ms", ctypes.c_double),
                ("cycles", ctypes.c_int64), ("checkpoints", ctypes.c_int32), ("status", ctypes.c_int32),
                ("sweep", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class ForceArgs(ctypes.Structure):
    """lulesh_force_args: device pointers for lulesh_calc_force_for_nodes_static."""
    _fields_ = [("num_elem", ctypes.c_int64), ("num_node", ctypes.c_int64),
                ("nodelist", ctypes.c_void_p), ("nodeElemStart", ctypes.c_void_p),
                ("nodeElemCount", ctypes.c_void_p), ("nodeElemCornerList", ctypes.c_void_p),
                ("x", ctypes.c_void_p), ("y", ctypes.c_void_p), ("z", ctypes.c_void_p),
                ("xd", ctypes.c_void_p), ("yd", ctypes.c_void_p), ("zd", ctypes.c_void_p),
                ("p", ctypes.c_void_p), ("q", ctypes.c_void_p), ("ss", ctypes.c_void_p),
                ("v", ctypes.c_void_p), ("volo", ctypes.c_void_p), ("elemMass", ctypes.c_void_p),
                ("hgcoef", ctypes.c_double), ("mode", ctypes.c_int32),
                ("fx", ctypes.c_void_p), ("fy", ctypes.c_void_p), ("fz", ctypes.c_void_p)]


_LIB = None


def library_path():
    """Path of the in-tree shared library built by lulesh.jl_gb300/build.py."""
    return os.environ.get("LULESH_GB300_LIB", os.path.join(_PKG, "lib", "liblulesh_gb300.so"))


def load_library():
    """Load liblulesh_gb300.so and declare its C signatures (no GPU needed)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError(
            f"liblulesh_gb300.so not found at {path}; build it with "
            "`python lulesh.jl_gb300/build.py` (the GPU path has no CPU fallback)")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    i32, i64, dbl = ctypes.c_int32, ctypes.c_int64, ctypes.c_double
    sig = {
        "lulesh_default_params": (None, [ctypes.POINTER(_Params), i32]),
        "lulesh_create": (ctypes.c_int, [ctypes.POINTER(_Params), ctypes.POINTER(P)]),
        "lulesh_destroy": (ctypes.c_int, [P]),
        "lulesh_time_increment": (ctypes.c_int, [P]),
        "lulesh_lagrange_leapfrog": (ctypes.c_int, [P]),
        "lulesh_run": (ctypes.c_int, [P, i64, ctypes.POINTER(_Scalars)]),
        "lulesh_get_scalars": (ctypes.c_int, [P, ctypes.POINTER(_Scalars)]),
        "lulesh_get_scalar": (ctypes.c_int, [P, i32, ctypes.POINTER(dbl)]),
        "lulesh_set_scalar": (ctypes.c_int, [P, i32, dbl]),
        "lulesh_field_length": (ctypes.c_int, [P, i32, ctypes.POINTER(i64)]),
        "lulesh_download_field": (ctypes.c_int, [P, i32, P, i64]),
        "lulesh_upload_field": (ctypes.c_int, [P, i32, P, i64]),
        "lulesh_verify": (ctypes.c_int, [P, ctypes.POINTER(dbl)]),
        "lulesh_sizes": (ctypes.c_int, [P, ctypes.POINTER(i64), ctypes.POINTER(i64)]),
        "lulesh_get_stream": (ctypes.c_int, [P, ctypes.POINTER(P)]),
        "lulesh_enable_timing": (ctypes.c_int, [P, i32]),
        "lulesh_kernel_times": (ctypes.c_int, [P, ctypes.POINTER(dbl), i32, ctypes.POINTER(i32)]),
        "lulesh_kernel_name": (ctypes.c_char_p, [i32]),
        "lulesh_status_string": (ctypes.c_char_p, [i32]),
        "lulesh_measure_fp64_peak": (ctypes.c_int, [i32, ctypes.POINTER(dbl), ctypes.POINTER(dbl)]),
        "lulesh_get_tuning": (ctypes.c_int, [P, ctypes.POINTER(Tuning)]),
        "lulesh_set_tuning": (ctypes.c_int, [P, ctypes.POINTER(Tuning)]),
        "lulesh_autotune": (ctypes.c_int, [P, i32, ctypes.POINTER(Tuning)]),
        "lulesh_ens_sedov_instances": (ctypes.c_int, [ctypes.c_uint64, i32, i32, i32, ctypes.POINTER(Instance)]),
        "lulesh_ens_create": (ctypes.c_int, [ctypes.POINTER(Instance), i32, i32, i32, ctypes.POINTER(P)]),
        "lulesh_ens_destroy": (ctypes.c_int, [P]),
        "lulesh_ens_run": (ctypes.c_int, [P, i64]),
        "lulesh_ens_reset": (ctypes.c_int, [P]),
        "lulesh_ens_sizes": (ctypes.c_int, [P, ctypes.POINTER(i32), ctypes.POINTER(i64), ctypes.POINTER(i64)]),
        "lulesh_ens_get_scalars": (ctypes.c_int, [P, i32, ctypes.POINTER(_Scalars)]),
        "lulesh_ens_field_length": (ctypes.c_int, [P, i32, i32, ctypes.POINTER(i64)]),
        "lulesh_ens_download_field": (ctypes.c_int, [P, i32, i32, P, i64]),
        "lulesh_ens_get_stream": (ctypes.c_int, [P, ctypes.POINTER(P)]),
        "lulesh_ens_get_tuning": (ctypes.c_int, [P, ctypes.POINTER(Tuning)]),
        "lulesh_ens_set_tuning": (ctypes.c_int, [P, ctypes.POINTER(Tuning)]),
        "lulesh_ens_autotune": (ctypes.c_int, [P, i32, ctypes.POINTER(Tuning)]),
        "lulesh_ens_partition": (ctypes.c_int, [ctypes.POINTER(Instance), i32, i32, ctypes.POINTER(i32)]),
        "lulesh_save_state": (ctypes.c_int, [P, ctypes.c_char_p]),
        "lulesh_load_state": (ctypes.c_int, [P, ctypes.c_char_p]),
        "lulesh_adj_create": (ctypes.c_int, [P, dbl, i32, ctypes.POINTER(P)]),
        "lulesh_adj_destroy": (ctypes.c_int, [P]),
        "lulesh_adj_set_seed": (ctypes.c_int, [P, i32, P, i64]),
        "lulesh_adj_clear_seeds": (ctypes.c_int, [P]),
        "lulesh_adj_loss": (ctypes.c_int, [P, ctypes.POINTER(dbl)]),
        "lulesh_adj_gradient": (ctypes.c_int, [P, i64, ctypes.POINTER(AdjResult)]),
        "lulesh_adj_get_gradient": (ctypes.c_int, [P, i32, P, i64]),
        "lulesh_adj_set_overlap": (ctypes.c_int, [P, i32]),
        "lulesh_create_blocks": (ctypes.c_int, [ctypes.POINTER(_Params), i32, ctypes.POINTER(P)]),
        "lulesh_block_map": (ctypes.c_int, [P, ctypes.POINTER(i32), P, P]),
        "lulesh_block_plan_sizes": (ctypes.c_int, [i32, i32, i32, ctypes.POINTER(i64)]),
        "lulesh_block_plan": (ctypes.c_int, [i32, i32, i32, P, P, P, P, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = L
    return L


def _check(rc, what):
    if rc == 0:
        return
    L = load_library()
    raise LuleshError(f"{what}: {L.lulesh_status_string(rc).decode()}", rc)


class LuleshProblem:
    """LuleshProblem (src/LULESH.jl:31-49) for one rank on one GPU.

    `devicetype` and `floattype` of the reference are fixed: device FP64.
    """

    def __init__(self, num_iters=10, structured=True, nx=45, nr=11, balance=1, cost=1,
                 mode=MODE_FAITHFUL, region_reps=False, keep_aux=False, device=0, region_seed=0,
                 blocks_per_edge=1):
        if not structured:
            raise LuleshError("Reading unstructured mesh is currently missing in the Julia version of LULESH.")
        self.num_iters = int(num_iters)
        self.structured = True
        self.nx = int(nx)
        self.nr = int(nr)
        self.balance = int(balance)
        self.cost = int(cost)
        self.mode = int(mode)
        self.region_reps = bool(region_reps)
        self.keep_aux = bool(keep_aux)
        self.device = int(device)
        self.region_seed = int(region_seed)
        # single rank: col = row = plane = 0, side = 1 (initMeshDecomp at one rank);
        # blocks_per_edge = tp > 1 builds the tp^3-rank decomposition of the
        # (tp*nx)^3 mesh as blocks of one handle (lulesh_create_blocks)
        self.col = self.row = self.plane = 0
        self.side = 1
        self.blocks_per_edge = int(blocks_per_edge)


class Domain:
    """The reference's Domain{Float64} (src/types.jl) held on the GPU.

    Field attributes (`domain.e`, `domain.x`, ...) return host numpy copies;
    assigning an array uploads it. Scalars (`domain.time`, `domain.hgcoef`,
    ...) read and write the handle's Domain scalars.
    """

    def __init__(self, prob):
        L = load_library()
        p = _Params()
        L.lulesh_default_params(ctypes.byref(p), prob.nx)
        p.nr, p.balance, p.cost, p.mode = prob.nr, prob.balance, prob.cost, prob.mode
        p.region_reps, p.keep_aux, p.device = int(prob.region_reps), int(prob.keep_aux), prob.device
        p.region_seed = prob.region_seed
        h = ctypes.c_void_p()
        tp = getattr(prob, "blocks_per_edge", 1)
        if tp > 1:
            _check(L.lulesh_create_blocks(ctypes.byref(p), tp, ctypes.byref(h)), "Domain(prob) in blocks")
        else:
            _check(L.lulesh_create(ctypes.byref(p), ctypes.byref(h)), "Domain(prob)")
        object.__setattr__(self, "_h", h)
        object.__setattr__(self, "_L", L)
        object.__setattr__(self, "prob", prob)
        ne, nn = ctypes.c_int64(), ctypes.c_int64()
        L.lulesh_sizes(h, ctypes.byref(ne), ctypes.byref(nn))
        object.__setattr__(self, "numElem", ne.value)
        object.__setattr__(self, "numNode", nn.value)
        object.__setattr__(self, "sizeX", prob.nx)

    @property
    def handle(self):
        return self._h

    def block_map(self):
        """(blocks per edge, whole-mesh element id of every packed element,
        whole-mesh node id of every packed node)."""
        tp = ctypes.c_int32()
        eg = np.empty(self.numElem, dtype=np.int32)
        ng = np.empty(self.numNode, dtype=np.int32)
        _check(self._L.lulesh_block_map(self._h, ctypes.byref(tp), eg.ctypes.data_as(ctypes.c_void_p),
                                        ng.ctypes.data_as(ctypes.c_void_p)), "block map")
        return tp.value, eg, ng

    def global_field(self, name):
        """A state or step field of a block mesh in the whole mesh's order
        (a node on a block face takes its first block's copy)."""
        _, eg, ng = self.block_map()
        v = self.field(name)
        ids = eg if v.size == self.numElem else ng
        out = np.empty(int(ids.max()) + 1, dtype=v.dtype)
        out[ids[::-1]] = v[::-1]  # the first copy wins
        return out

    def close(self):
        if self._h:
            self._L.lulesh_destroy(self._h)
            object.__setattr__(self, "_h", None)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def field(self, name, out=None):
        """A copy of the field on the host; with `out` (a C-contiguous array of
        the field's dtype and length, e.g. in pinned memory) the copy lands
        there directly and `out` is returned."""
        fid, dt = FIELDS[name]
        n = ctypes.c_int64()
        _check(self._L.lulesh_field_length(self._h, fid, ctypes.byref(n)), f"length of {name}")
        if out is None:
            out = np.empty(n.value, dtype=dt)
        elif (not isinstance(out, np.ndarray) or out.dtype != np.dtype(dt) or out.size != n.value
              or not out.flags.c_contiguous or not out.flags.writeable):
            raise ValueError(f"out must be a writeable C-contiguous {np.dtype(dt)} array of {n.value} values")
        _check(self._L.lulesh_download_field(self._h, fid, out.ctypes.data_as(ctypes.c_void_p), n.value),
               f"download {name}")
        return out

    def set_field(self, name, values):
        fid, dt = FIELDS[name]
        arr = np.ascontiguousarray(values, dtype=dt)
        _check(self._L.lulesh_upload_field(self._h, fid, arr.ctypes.data_as(ctypes.c_void_p), arr.size),
               f"upload {name}")

    def scalars(self):
        s = _Scalars()
        _check(self._L.lulesh_get_scalars(self._h, ctypes.byref(s)), "scalars")
        return {k: getattr(s, k) for k, _ in _Scalars._fields_}

    def stream(self):
        s = ctypes.c_void_p()
        _check(self._L.lulesh_get_stream(self._h, ctypes.byref(s)), "stream")
        return s.value

    def enable_timing(self, on=True):
        _check(self._L.lulesh_enable_timing(self._h, int(on)), "timing")

    def kernel_times(self):
        ms = (ctypes.c_double * 16)()
        n = ctypes.c_int32()
        _check(self._L.lulesh_kernel_times(self._h, ms, 16, ctypes.byref(n)), "kernel times")
        return {self._L.lulesh_kernel_name(i).decode(): ms[i] for i in range(n.value)}

    def tuning(self):
        t = Tuning()
        _check(self._L.lulesh_get_tuning(self._h, ctypes.byref(t)), "tuning")
        return t.as_dict()

    def set_tuning(self, **blocks):
        t = Tuning()
        self._L.lulesh_get_tuning(self._h, ctypes.byref(t))
        for k, v in blocks.items():
            setattr(t, k, int(v))
        _check(self._L.lulesh_set_tuning(self._h, ctypes.byref(t)), "set tuning")

    def autotune(self, cycles=3):
        """Times each kernel's candidate block sizes on this problem; the state is kept."""
        t = Tuning()
        _check(self._L.lulesh_autotune(self._h, int(cycles), ctypes.byref(t)), "autotune")
        return t.as_dict()

    def save_state(self, path):
        """Write the step state (state fields and Domain scalars) to `path`."""
        _check(self._L.lulesh_save_state(self._h, os.fsencode(path)), f"save state to {path}")

    def load_state(self, path):
        """Load a state file written for the same problem; the run then
        continues as the saved one would have."""
        _check(self._L.lulesh_load_state(self._h, os.fsencode(path)), f"load state from {path}")

    def __getattr__(self, name):
        if name in FIELDS:
            return self.field(name)
        if name in SCALARS:
            v = ctypes.c_double()
            _check(self._L.lulesh_get_scalar(self._h, SCALARS[name], ctypes.byref(v)), name)
            return int(v.value) if name == "cycle" else v.value
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in FIELDS:
            self.set_field(name, value)
        elif name in SCALARS:
            _check(self._L.lulesh_set_scalar(self._h, SCALARS[name], float(value)), name)
        else:
            object.__setattr__(self, name, value)


def _raise_step(domain, rc):
    s = domain.scalars()
    msg = _MESSAGES.get((rc, s["site"] if rc == 1 else 0), None)
    if msg is None:
        msg = load_library().lulesh_status_string(rc).decode()
    raise LuleshError(msg, rc, s["site"])


def timeIncrement(domain):
    """timeIncrement!(domain), src/domain.jl:920-961."""
    _check(domain._L.lulesh_time_increment(domain._h), "timeIncrement!")


def lagrangeLeapFrog(domain):
    """lagrangeLeapFrog(domain), src/domain.jl:3067-3080 (one step on the GPU)."""
    rc = domain._L.lulesh_lagrange_leapfrog(domain._h)
    if rc:
        _raise_step(domain, rc)


def run(domain, num_iters):
    """The examples/benchmark.jl:82-98 loop, device-resident; returns the scalars."""
    s = _Scalars()
    rc = domain._L.lulesh_run(domain._h, int(num_iters), ctypes.byref(s))
    if rc:
        _raise_step(domain, rc)
    return {k: getattr(s, k) for k, _ in _Scalars._fields_}


def verify(domain):
    """(origin energy, MaxAbsDiff, TotalAbsDiff, MaxRelDiff), src/utils.jl:124-158."""
    out = (ctypes.c_double * 4)()
    _check(domain._L.lulesh_verify(domain._h, out), "verify")
    return tuple(out)


def verifyAndWriteFinalOutput(elapsed_time, domain, nx, numRanks=1, file=None):
    """Prints the reference's final report (src/utils.jl:124-164); returns its numbers."""
    import sys
    f = file or sys.stdout
    e0, maxabs, total, maxrel = verify(domain)
    cyc = domain.cycle
    grind1 = ((elapsed_time * 1e6) / cyc) / (nx * nx * nx) if cyc else float("nan")
    grind2 = ((elapsed_time * 1e6) / cyc) / (nx * nx * nx * numRanks) if cyc else float("nan")
    print("Run completed:", file=f)
    print(f"   Problem size        =  {nx}", file=f)
    print(f"   MPI tasks           =  {numRanks}", file=f)
    print(f"   Iteration count     =  {cyc}", file=f)
    print(f"   Final Origin Energy =  {e0:.6e}", file=f)
    print("   Testing Plane 0 of Energy Array on rank 0:", file=f)
    print(f"        MaxAbsDiff   = {maxabs:.6e}", file=f)
    print(f"        TotalAbsDiff = {total:.6e}", file=f)
    print(f"        MaxRelDiff   = {maxrel:.6e}", file=f)
    print(f"\nElapsed time         = {elapsed_time:.2f} (s)", file=f)
    # the reference prints elapsed_time where it means grindTime2 (src/utils.jl:162)
    print(f"Grind time (us/z/c)  =  {grind1:.8f}  (per dom)  ({elapsed_time:.8f} overall)", file=f)
    print(f"FOM                  = {1000.0 / grind2:.8f} (z/s)\n", file=f)
    return {"origin_energy": e0, "MaxAbsDiff": maxabs, "TotalAbsDiff": total, "MaxRelDiff": maxrel,
            "cycle": cyc, "grind_us": grind2, "fom_kzs": 1000.0 / grind2}


def block_plan(nx, blocks_per_edge, mode=MODE_FAITHFUL):
    """The tp^3 decomposition of the (tp*nx)^3 mesh and its halo plan,
    computed on the host (no GPU): packed -> whole-mesh element and node ids,
    and per ghost slot the packed element (delv) or corner-force slot
    c*E + e (corners) it copies and the block that holds the slot."""
    L = load_library()
    sizes = (ctypes.c_int64 * 5)()
    _check(L.lulesh_block_plan_sizes(int(nx), int(blocks_per_edge), int(mode), sizes), "block plan sizes")
    E, N, gd, gc, ncl = (int(v) for v in sizes)
    out = {"E": E, "N": N, "corner_list_entries": ncl,
           "elem_global": np.empty(E, np.int32), "node_global": np.empty(N, np.int32),
           "halo_delv_src": np.empty(gd, np.int32), "halo_delv_dst": np.empty(gd, np.int32),
           "halo_corner_src": np.empty(gc, np.int32), "halo_corner_dst": np.empty(gc, np.int32)}
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    _check(L.lulesh_block_plan(int(nx), int(blocks_per_edge), int(mode), ptr(out["elem_global"]),
                               ptr(out["node_global"]), ptr(out["halo_delv_src"]), ptr(out["halo_delv_dst"]),
                               ptr(out["halo_corner_src"]), ptr(out["halo_corner_dst"])), "block plan")
    return out


def sedov_instances(seed=0xC4, n=256, nx_min=16, nx_max=64):
    """The seeded instance draw of lulesh_ens_sedov_instances (list of dicts)."""
    L = load_library()
    arr = (Instance * n)()
    _check(L.lulesh_ens_sedov_instances(int(seed), int(n), int(nx_min), int(nx_max), arr), "instances")
    return [{k: getattr(a, k) for k, _ in Instance._fields_} for a in arr]


def _instance_array(instances):
    """lulesh_instance array; missing keys take the reference's defaults."""
    arr = (Instance * max(1, len(instances)))()
    for a, spec in zip(arr, instances):
        a.nx = int(spec["nx"])
        a.nr = int(spec.get("nr", 11))
        a.balance = int(spec.get("balance", 1))
        a.cost = int(spec.get("cost", 1))
        a.einit = float(spec.get("einit", 0.0))
        a.hgcoef = float(spec.get("hgcoef", 3.0))
        a.region_seed = int(spec.get("region_seed", 0))
    return arr


def partition(instances, parts):
    """lulesh_ens_partition: the part (GPU rank) of every instance, balancing
    the cost nx^3 greedily, largest first. Deterministic."""
    L = load_library()
    n = len(instances)
    out = (ctypes.c_int32 * max(1, n))()
    _check(L.lulesh_ens_partition(_instance_array(instances), n, int(parts), out), "partition")
    return [int(out[i]) for i in range(n)]


def shard(instances, world, rank):
    """The instances rank `rank` of `world` advances (indices and specs)."""
    part = partition(instances, world)
    idx = [i for i, p in enumerate(part) if p == rank]
    return idx, [instances[i] for i in idx]


class Ensemble:
    """Many independent Sedov problems advanced together on one GPU.

    `instances` is a list of dicts with the lulesh_instance keys (nx, nr,
    balance, cost, einit, hgcoef, region_seed); missing keys take the
    reference's defaults. `run(num_iters)` runs examples/benchmark.jl's loop
    for every instance at once, device-resident.
    """

    def __init__(self, instances, mode=MODE_FAITHFUL, device=0):
        L = load_library()
        n = len(instances)
        arr = _instance_array(instances)
        h = ctypes.c_void_p()
        _check(L.lulesh_ens_create(arr, n, int(mode), int(device), ctypes.byref(h)), "ensemble create")
        self._L, self._h, self.n = L, h, n
        self.instances = [dict(s) for s in instances]
        c = ctypes.c_int32()
        te, tn = ctypes.c_int64(), ctypes.c_int64()
        L.lulesh_ens_sizes(h, ctypes.byref(c), ctypes.byref(te), ctypes.byref(tn))
        self.total_elem, self.total_node = te.value, tn.value

    def close(self):
        if self._h:
            self._L.lulesh_ens_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, num_iters):
        rc = self._L.lulesh_ens_run(self._h, int(num_iters))
        if rc:
            raise LuleshError(f"ensemble run: {self._L.lulesh_status_string(rc).decode()}", rc)

    def reset(self):
        _check(self._L.lulesh_ens_reset(self._h), "ensemble reset")

    def scalars(self, i):
        s = _Scalars()
        _check(self._L.lulesh_ens_get_scalars(self._h, int(i), ctypes.byref(s)), "ensemble scalars")
        return {k: getattr(s, k) for k, _ in _Scalars._fields_}

    def field(self, i, name):
        fid, dt = FIELDS[name]
        n = ctypes.c_int64()
        _check(self._L.lulesh_ens_field_length(self._h, int(i), fid, ctypes.byref(n)), f"length of {name}")
        out = np.empty(n.value, dtype=dt)
        _check(self._L.lulesh_ens_download_field(self._h, int(i), fid, out.ctypes.data_as(ctypes.c_void_p),
                                                 n.value), f"download {name}")
        return out

    def stream(self):
        s = ctypes.c_void_p()
        _check(self._L.lulesh_ens_get_stream(self._h, ctypes.byref(s)), "stream")
        return s.value

    def tuning(self):
        t = Tuning()
        _check(self._L.lulesh_ens_get_tuning(self._h, ctypes.byref(t)), "tuning")
        return t.as_dict()

    def set_tuning(self, **blocks):
        t = Tuning()
        self._L.lulesh_ens_get_tuning(self._h, ctypes.byref(t))
        for k, v in blocks.items():
            setattr(t, k, int(v))
        _check(self._L.lulesh_ens_set_tuning(self._h, ctypes.byref(t)), "set tuning")

    def autotune(self, cycles=3):
        """Picks block sizes on this ensemble, then returns it to its initial state."""
        t = Tuning()
        _check(self._L.lulesh_ens_autotune(self._h, int(cycles), ctypes.byref(t)), "autotune")
        return t.as_dict()


# The state a cycle maps to the next one (node then element fields).
STATE_FIELDS = ("x", "y", "z", "xd", "yd", "zd", "e", "p", "q", "v", "ss")


class Adjoint:
    """Reverse-mode gradient of a run of a Domain (lulesh_adj_* of the C ABI).

    The reference differentiates `lagrangeLeapFrog` with Enzyme
    (examples/benchmark.jl:48-52, 85-86: `autodiff(lagrangeLeapFrog,
    Duplicated(domain, shadow))`); this is a hand-written adjoint of whole runs.
    The default objective after the run is the energy within `radius` of the
    origin (element internal energy times mass, plus nodal kinetic energy,
    masked by the initial mesh); `set_seed` replaces it with linear weights on
    state fields. `gradient(n)` advances the domain by up to n cycles and
    returns the objective; `grad(name)` is then the gradient w.r.t. that
    field's value before the run and `result.grad_hgcoef` w.r.t. hgcoef.
    """

    def __init__(self, domain, radius=0.3, checkpoint_every=20):
        L = load_library()
        h = ctypes.c_void_p()
        _check(L.lulesh_adj_create(domain.handle, float(radius), int(checkpoint_every), ctypes.byref(h)),
               "adjoint")
        self._L, self._h, self.domain = L, h, domain
        self.result = None

    def close(self):
        if self._h:
            self._L.lulesh_adj_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_seed(self, name, weights):
        fid, _ = FIELDS[name]
        w = np.ascontiguousarray(weights, dtype=np.float64)
        _check(self._L.lulesh_adj_set_seed(self._h, fid, w.ctypes.data_as(ctypes.c_void_p), w.size),
               f"seed {name}")

    def clear_seeds(self):
        _check(self._L.lulesh_adj_clear_seeds(self._h), "clear seeds")

    def set_overlap(self, mode):
        """How the reverse sweep runs: False/0 each segment's recompute and
        then its transpose; True/1 (the default) the recompute of one segment
        overlapped with the transpose of the next, on two tapes where the
        second fits, else on one; 2 overlapped on one tape. result.sweep
        tells which a gradient took (0, 1 two tapes, 2 one tape)."""
        m = int(mode)
        if m not in (0, 1, 2):
            raise ValueError("overlap mode is 0, 1 or 2")
        _check(self._L.lulesh_adj_set_overlap(self._h, m), "overlap")

    def loss(self):
        x = ctypes.c_double()
        _check(self._L.lulesh_adj_loss(self._h, ctypes.byref(x)), "loss")
        return x.value

    def gradient(self, num_cycles):
        r = AdjResult()
        rc = self._L.lulesh_adj_gradient(self._h, int(num_cycles), ctypes.byref(r))
        if rc:
            _raise_step(self.domain, rc)
        self.result = r
        return r.loss

    def grad(self, name):
        fid, _ = FIELDS[name]
        n = self.domain.numNode if fid >= 32 else self.domain.numElem
        out = np.empty(n)
        _check(self._L.lulesh_adj_get_gradient(self._h, fid, out.ctypes.data_as(ctypes.c_void_p), n),
               f"gradient {name}")
        return out


def read_state(path, verify=True):
    """Host-side reader of a lulesh_save_state file (no GPU needed): a dict
    with the problem header, the Domain scalars by name and the state fields
    as numpy arrays. Checks the magic and, with `verify`, the trailing FNV-1a
    hash (a byte-serial loop in Python: about a second per 10 MB; the
    library's own load always checks it)."""
    with open(path, "rb") as f:
        raw = f.read()
    if raw[:8] != b"LULESHS1":
        raise ValueError(f"{path}: not a LULESH state file")
    body, (stored,) = raw[8:-8], np.frombuffer(raw[-8:], dtype="<u8")
    if verify:
        h = 1469598103934665603
        for b in body:
            h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
        if h != int(stored):
            raise ValueError(f"{path}: hash mismatch")
    head = np.frombuffer(body, dtype="<i4", count=6)
    sizes = np.frombuffer(body, dtype="<i8", count=2, offset=24)
    ns, nf = np.frombuffer(body, dtype="<i4", count=2, offset=40)
    off = 48
    sc = np.frombuffer(body, dtype="<f8", count=int(ns), offset=off)
    off += 8 * int(ns)
    names = {v[0]: k for k, v in FIELDS.items()}
    fields = {}
    for _ in range(int(nf)):
        fid = int(np.frombuffer(body, dtype="<i4", count=1, offset=off)[0])
        n = int(np.frombuffer(body, dtype="<i8", count=1, offset=off + 4)[0])
        fields[names[fid]] = np.frombuffer(body, dtype="<f8", count=n, offset=off + 12).copy()
        off += 12 + 8 * n
    inv = {i: k for k, i in SCALARS.items()}
    return {"version": int(head[0]), "nx": int(head[1]), "nr": int(head[2]), "balance": int(head[3]),
            "cost": int(head[4]), "mode": int(head[5]), "numElem": int(sizes[0]), "numNode": int(sizes[1]),
            "scalars": {inv[i]: float(v) for i, v in enumerate(sc)}, "fields": fields}
