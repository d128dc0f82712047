"""The region cost model (LULESH 2.0's rep loop in EvalEOSForElems, on the
problem's own region layout): with region_reps on, each element's EOS is
evaluated regReps times, in region order. The reference computes regReps but
never applies them, so results must not change: bitwise equal to the run
without reps, and within the parity bar of the oracle for an unbalanced
layout (balance=4, cost=2)."""
import numpy as np
import pytest

from conftest import field_floor, rel_err

pytestmark = pytest.mark.gpu

STATE = ["e", "p", "q", "v", "ss", "x", "y", "z", "xd", "yd", "zd"]


def run(L, nx, cycles, reps, balance=4, cost=2, mode=0, aux=False):
    g = L.Domain(L.LuleshProblem(nx=nx, nr=11, balance=balance, cost=cost, mode=mode,
                                 region_reps=reps, keep_aux=aux))
    L.run(g, cycles)
    return g


@pytest.mark.parametrize("mode", [0, 7])
def test_region_reps_leave_results_unchanged(gpu_lib, mode):
    L = gpu_lib
    a = run(L, 20, 60, False, mode=mode)
    b = run(L, 20, 60, True, mode=mode)
    assert a.cycle == b.cycle == 60
    for s in ("time", "deltatime", "dtcourant", "dthydro"):
        assert getattr(a, s) == getattr(b, s), s
    for f in STATE:
        assert np.array_equal(a.field(f), b.field(f)), f


def test_region_reps_stepwise_and_aux(gpu_lib):
    L = gpu_lib
    a = run(L, 12, 25, False, aux=True)
    g = L.Domain(L.LuleshProblem(nx=12, nr=11, balance=4, cost=2, region_reps=True, keep_aux=True))
    for _ in range(25):
        L.timeIncrement(g)
        L.lagrangeLeapFrog(g)
    for f in STATE + ["ql", "qq", "fx", "xdd"]:
        assert np.array_equal(a.field(f), g.field(f)), f


def test_unbalanced_regions_match_oracle(gpu_lib, oracle_mod):
    L = gpu_lib
    nx, cycles = 16, 40
    g = run(L, nx, cycles, True)
    o = oracle_mod.OracleDomain(nx, nr=11, balance=4, cost=2)
    assert o.run(cycles) == 0
    assert g.cycle == o.get("cycle")
    assert g.time == pytest.approx(o.get("time"), rel=1e-12)
    for f in ["regElemlist", "regReps", "regElemSize", "regNumList"]:
        assert np.array_equal(g.field(f), o.field(f)), f
    for f in STATE:
        b = o.field(f)
        assert rel_err(g.field(f), b, field_floor(f, b)) <= 1e-8, f
