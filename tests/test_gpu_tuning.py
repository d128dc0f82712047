"""The launch choices the autotuner makes change no result: block sizes and
the fusion split of the force geometry (stored by k_kinematics, or formed in
k_force) give bitwise the same states and gradients, also when the split
changes in the middle of a run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE = ["e", "p", "q", "v", "ss", "x", "y", "z", "xd", "yd", "zd"]


def same_state(a, b):
    for f in STATE + ["vdov", "arealg", "delv"]:
        assert np.array_equal(a.field(f), b.field(f)), f
    for s in ["time", "deltatime", "dtcourant", "dthydro", "cycle"]:
        assert getattr(a, s) == getattr(b, s), s


@pytest.mark.parametrize("mode", [0, 7])
def test_geometry_split_is_bitwise_neutral(gpu_lib, mode):
    L = gpu_lib
    a = L.Domain(L.LuleshProblem(nx=12, mode=mode))
    b = L.Domain(L.LuleshProblem(nx=12, mode=mode))
    b.set_tuning(geometry=1, force_block=256, kin_block=64)
    assert b.tuning()["geometry"] == 1 and a.tuning()["geometry"] == 0
    L.run(a, 30)
    L.run(b, 30)
    same_state(a, b)
    # switch both splits mid-run and continue step by step (the stored split
    # has to form the geometry of positions the inline split moved)
    a.set_tuning(geometry=1)
    b.set_tuning(geometry=0)
    for _ in range(10):
        L.timeIncrement(a)
        L.lagrangeLeapFrog(a)
        L.timeIncrement(b)
        L.lagrangeLeapFrog(b)
    same_state(a, b)
    L.run(a, 60)
    L.run(b, 60)
    same_state(a, b)


def test_geometry_split_in_the_ensemble(gpu_lib):
    L = gpu_lib
    inst = [{"nx": 5, "nr": 11}, {"nx": 9, "nr": 1, "hgcoef": 2.2}, {"nx": 3, "einit": 1e5}]
    a, b = L.Ensemble(inst), L.Ensemble(inst)
    b.set_tuning(geometry=1)
    a.run(20)
    b.run(20)
    a.set_tuning(geometry=1)
    b.set_tuning(geometry=0)
    a.run(45)
    b.run(45)
    for i in range(len(inst)):
        for f in STATE:
            assert np.array_equal(a.field(i, f), b.field(i, f)), (i, f)
        assert a.scalars(i) == b.scalars(i)


def test_geometry_split_in_the_adjoint(gpu_lib):
    """The adjoint's untaped forward segments run the domain's split; its
    taping kernels always use the stored geometry. The gradient is the same."""
    L = gpu_lib
    res = []
    for geo in (0, 1):
        g = L.Domain(L.LuleshProblem(nx=8))
        L.run(g, 5)
        g.set_tuning(geometry=geo)
        adj = L.Adjoint(g, checkpoint_every=6)
        loss = adj.gradient(25)
        res.append((loss, adj.result.grad_hgcoef, {f: adj.grad(f) for f in STATE}, g.field("e")))
        adj.close()
        g.close()
    assert res[0][0] == res[1][0] and res[0][1] == res[1][1]
    for f in STATE:
        assert np.array_equal(res[0][2][f], res[1][2][f]), f
    assert np.array_equal(res[0][3], res[1][3])


def test_autotune_reports_a_split_and_keeps_results(gpu_lib):
    L = gpu_lib
    a = L.Domain(L.LuleshProblem(nx=20))
    b = L.Domain(L.LuleshProblem(nx=20))
    L.run(a, 5)
    L.run(b, 5)
    chosen = a.autotune(cycles=2)
    assert chosen["geometry"] in (0, 1)
    assert chosen["force_block"] in (64, 128, 256) and chosen["kin_block"] in (64, 128, 256)
    L.run(a, 40)
    L.run(b, 40)
    same_state(a, b)
