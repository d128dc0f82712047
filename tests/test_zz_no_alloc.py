"""The allocation-free force entry point, for callers that cannot let the
library allocate device memory (their device arrays come from their own
memory pool, or every byte of device memory is budgeted up front).

Checked through the C ABI with caller-owned device buffers, on two calls in a
row, against two independent results:
  * the forces the regular step computes from the same state
    (lulesh_lagrange_leapfrog keeps fx, fy, fz with keep_aux);
  * the CPU oracle's calcForceForNodes on the same state.
Both at 1e-8 relative (floor 1e-7 of the field's largest magnitude: nodal
sums with cancellation), in the modes that change the force arithmetic, up to
the documented limit of 32,768 elements. The volume checks are provoked on the
host (an inverted element, a negative relative volume).
"""
import ctypes

import numpy as np
import pytest

from conftest import field_floor, rel_err

pytestmark = pytest.mark.gpu

P = ctypes.c_void_p
INDEX = ("nodelist", "nodeElemStart", "nodeElemCount", "nodeElemCornerList")
STATE = ("x", "y", "z", "xd", "yd", "zd", "p", "q", "ss", "v", "volo", "elemMass")
MAX_ELEMS = 32768  # LULESH_STATIC_MAX_ELEMS


def _entry(gpu_lib):
    fn = gpu_lib.load_library().lulesh_calc_force_for_nodes_static
    fn.argtypes = [ctypes.POINTER(gpu_lib.ForceArgs), P, ctypes.POINTER(ctypes.c_int32)]
    fn.restype = ctypes.c_int
    return fn


def _args(gpu_lib, g, dev, mode):
    a = gpu_lib.ForceArgs(num_elem=g.numElem, num_node=g.numNode, hgcoef=g.hgcoef, mode=mode)
    for n in INDEX + STATE + ("fx", "fy", "fz"):
        setattr(a, n, dev[n].data_ptr())
    return a


def _upload(g, dev, overrides=None):
    import torch
    for n in STATE:
        v = g.field(n) if not overrides or n not in overrides else overrides[n]
        dev[n] = torch.from_numpy(np.ascontiguousarray(v)).cuda()
    for n in ("fx", "fy", "fz"):
        dev[n] = torch.full((g.numNode,), np.nan, dtype=torch.float64, device="cuda")


def _close(got, ref, n):
    floor = max(field_floor(n, ref), 1e-7 * float(np.abs(ref).max()))
    return rel_err(got, ref, floor)


@pytest.mark.parametrize("nx", [14, 32])
@pytest.mark.parametrize("mode", [0, 1, 2, 7])
def test_static_forces_match_step_and_oracle(gpu_lib, oracle_mod, nx, mode):
    import torch
    L = gpu_lib
    fn = _entry(gpu_lib)
    g = L.Domain(L.LuleshProblem(nx=nx, mode=mode, keep_aux=True))
    assert g.numElem <= MAX_ELEMS
    o = oracle_mod.OracleDomain(nx, mode=mode)
    L.run(g, 25)  # stress and hourglass forces are both active by now
    dev = {n: torch.from_numpy(g.field(n)).cuda() for n in INDEX}
    stream = P(torch.cuda.current_stream().cuda_stream)
    free_before = None
    for call in range(2):
        _upload(g, dev)
        a = _args(gpu_lib, g, dev, mode)
        torch.cuda.synchronize()
        if call == 1:
            free_before = torch.cuda.mem_get_info()[0]
        site = ctypes.c_int32(-1)
        rc = fn(ctypes.byref(a), stream, ctypes.byref(site))
        assert rc == 0 and site.value == 0, (call, rc, site.value)
        if call == 1:
            # the second call on this device commits no device memory
            assert torch.cuda.mem_get_info()[0] == free_before
        got = {n: dev[n].cpu().numpy() for n in ("fx", "fy", "fz")}
        # the oracle's calcForceForNodes on the same state
        for n in ("x", "y", "z", "xd", "yd", "zd", "p", "q", "ss", "v"):
            o.set_field(n, g.field(n))
        assert o.L.ora_force_for_nodes(o.h) == 0
        for n in ("fx", "fy", "fz"):
            assert _close(got[n], o.field(n), n) <= 1e-8, ("oracle", call, n)
        # the existing entry point computes its forces from this same state
        L.timeIncrement(g)
        L.lagrangeLeapFrog(g)
        for n in ("fx", "fy", "fz"):
            assert _close(got[n], g.field(n), n) <= 1e-8, ("step", call, n)
    g.close()
    o.close()


@pytest.mark.parametrize("case", ["inverted", "negative_volume"])
def test_static_forces_volume_checks(gpu_lib, case):
    """An element dragged through its neighbour fails the detJ check
    (site EARLY, src/domain.jl:1104); a negative relative volume fails the
    hourglass control's v check (site HOURGLASS, src/domain.jl:1727). Both
    states are made on the host; the kernel only reads them."""
    import torch
    L = gpu_lib
    fn = _entry(gpu_lib)
    g = L.Domain(L.LuleshProblem(nx=4))
    dev = {n: torch.from_numpy(g.field(n)).cuda() for n in INDEX}
    if case == "inverted":
        x = g.field("x")
        x[1] = -0.9
        _upload(g, dev, {"x": x})
        want = 1  # LULESH_SITE_EARLY
    else:
        v = g.field("v")
        v[5] = -1.0
        _upload(g, dev, {"v": v})
        want = 2  # LULESH_SITE_HOURGLASS
    a = _args(gpu_lib, g, dev, 0)
    torch.cuda.synchronize()
    site = ctypes.c_int32(-1)
    rc = fn(ctypes.byref(a), P(torch.cuda.current_stream().cuda_stream), ctypes.byref(site))
    assert rc == 1 and site.value == want
    # the status word is cleared by the next call: a good state passes again
    _upload(g, dev)
    a = _args(gpu_lib, g, dev, 0)
    torch.cuda.synchronize()
    rc = fn(ctypes.byref(a), P(torch.cuda.current_stream().cuda_stream), ctypes.byref(site))
    assert rc == 0 and site.value == 0
    g.close()


def test_static_forces_reject_oversize(gpu_lib):
    fn = _entry(gpu_lib)
    a = gpu_lib.ForceArgs(num_elem=MAX_ELEMS + 1, num_node=10, hgcoef=3.0, mode=0)
    for n in INDEX + STATE + ("fx", "fy", "fz"):
        setattr(a, n, 8)  # never dereferenced: the size check comes first
    site = ctypes.c_int32(0)
    assert fn(ctypes.byref(a), None, ctypes.byref(site)) == 6
