"""The allocation-free force entry point, for callers that cannot let the
library allocate device memory (their device arrays come from their own
memory pool). It is checked against the forces the regular step computes
(lulesh_lagrange_leapfrog keeps fx, fy, fz with keep_aux) on two calls in a
row, through the C ABI with caller-owned device buffers.
"""
import ctypes

import numpy as np
import pytest

from conftest import field_floor, rel_err

pytestmark = pytest.mark.gpu

P = ctypes.c_void_p


class ForceArgs(ctypes.Structure):
    # lulesh_force_args in include/lulesh_gb300.h
    _fields_ = [("num_elem", ctypes.c_int64), ("num_node", ctypes.c_int64),
                ("nodelist", P), ("nodeElemStart", P), ("nodeElemCount", P), ("nodeElemCornerList", P),
                ("x", P), ("y", P), ("z", P), ("xd", P), ("yd", P), ("zd", P),
                ("p", P), ("q", P), ("ss", P), ("v", P), ("volo", P), ("elemMass", P),
                ("hgcoef", ctypes.c_double), ("mode", ctypes.c_int32),
                ("fx", P), ("fy", P), ("fz", P)]


INDEX = ("nodelist", "nodeElemStart", "nodeElemCount", "nodeElemCornerList")
STATE = ("x", "y", "z", "xd", "yd", "zd", "p", "q", "ss", "v", "volo", "elemMass")


def _entry(gpu_lib):
    fn = gpu_lib.load_library().lulesh_calc_force_for_nodes_static
    fn.argtypes = [ctypes.POINTER(ForceArgs), P, ctypes.POINTER(ctypes.c_int32)]
    fn.restype = ctypes.c_int
    return fn


@pytest.mark.parametrize("mode", [0, 7])
def test_static_forces_match_step_forces(gpu_lib, mode):
    import torch
    L = gpu_lib
    fn = _entry(gpu_lib)
    g = L.Domain(L.LuleshProblem(nx=14, mode=mode, keep_aux=True))
    L.run(g, 25)  # stress and hourglass forces are both active by now
    dev = {n: torch.from_numpy(g.field(n)).cuda() for n in INDEX}
    for call in range(2):
        for n in STATE:
            dev[n] = torch.from_numpy(g.field(n)).cuda()
        for n in ("fx", "fy", "fz"):
            dev[n] = torch.full((g.numNode,), np.nan, dtype=torch.float64, device="cuda")
        a = ForceArgs(num_elem=g.numElem, num_node=g.numNode, hgcoef=g.hgcoef, mode=mode)
        for n in INDEX + STATE + ("fx", "fy", "fz"):
            setattr(a, n, dev[n].data_ptr())
        torch.cuda.synchronize()
        site = ctypes.c_int32(-1)
        rc = fn(ctypes.byref(a), P(torch.cuda.current_stream().cuda_stream), ctypes.byref(site))
        assert rc == 0 and site.value == 0, (call, rc, site.value)
        # the existing entry point computes its forces from this same state
        L.timeIncrement(g)
        L.lagrangeLeapFrog(g)
        for n in ("fx", "fy", "fz"):
            ref = g.field(n)
            got = dev[n].cpu().numpy()
            floor = max(field_floor(n, ref), 1e-7 * float(np.abs(ref).max()))
            assert rel_err(got, ref, floor) <= 1e-8, (call, n)
    g.close()


def test_static_forces_reject_oversize(gpu_lib):
    fn = _entry(gpu_lib)
    a = ForceArgs(num_elem=32768 + 1, num_node=10, hgcoef=3.0, mode=0)
    for n in INDEX + STATE + ("fx", "fy", "fz"):
        setattr(a, n, 8)  # never dereferenced: the size check comes first
    site = ctypes.c_int32(0)
    assert fn(ctypes.byref(a), None, ctypes.byref(site)) == 6
