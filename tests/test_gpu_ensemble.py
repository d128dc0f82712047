"""The batched ensemble: every instance against the oracle and against the
single-problem GPU path, plus reset, autotuning and the seeded draw."""
import math

import numpy as np
import pytest

from conftest import field_floor, rel_err

STATE = ["e", "p", "q", "v", "ss", "x", "y", "z", "xd", "yd", "zd"]

# Uneven sizes, energies and hourglass coefficients; nr = 1 and 11.
SMALL = [
    {"nx": 5, "nr": 11, "hgcoef": 3.0, "einit": 0.0},
    {"nx": 9, "nr": 1, "hgcoef": 2.2, "einit": 1.7 * 3.948746e7 * (9 / 45) ** 3},
    {"nx": 3, "nr": 11, "hgcoef": 3.9, "einit": 0.6 * 3.948746e7 * (3 / 45) ** 3},
    {"nx": 12, "nr": 11, "hgcoef": 2.6, "einit": 0.0},
    {"nx": 7, "nr": 1, "hgcoef": 0.0, "einit": 0.0},
]


def test_instance_draw_is_seeded_and_in_range(gpu_lib):
    a = gpu_lib.sedov_instances(0xC4, 256, 16, 64)
    b = gpu_lib.sedov_instances(0xC4, 256, 16, 64)
    assert a == b
    assert a != gpu_lib.sedov_instances(0xC5, 256, 16, 64)
    for s in a:
        assert 16 <= s["nx"] <= 64
        assert 2.0 <= s["hgcoef"] <= 4.0
        assert s["nr"] in (1, 11)
        f = s["einit"] / (3.948746e7 * (s["nx"] / 45.0) ** 3)
        assert 0.5 <= f <= 2.0
    assert 60 < sum(s["nr"] == 11 for s in a) < 196
    assert len({s["nx"] for s in a}) > 30


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 7])
def test_ensemble_matches_oracle(gpu_lib, oracle_mod, mode):
    ens = gpu_lib.Ensemble(SMALL, mode=mode)
    iters = 60
    ens.run(iters)
    for i, spec in enumerate(SMALL):
        o = oracle_mod.OracleDomain(spec["nx"], nr=spec["nr"], mode=mode)
        o.set("hgcoef", spec["hgcoef"])
        if spec["einit"] > 0:
            o.set_einit(spec["einit"])
        assert o.run(iters) == 0
        s = ens.scalars(i)
        # small instances reach stoptime before iters cycles (3^3: 16 cycles)
        assert s["cycle"] == o.get("cycle"), i
        assert s["cycle"] == iters or o.get("time") >= o.get("stoptime"), i
        assert s["time"] == pytest.approx(o.get("time"), rel=1e-12), i
        for f in STATE:
            a, b = ens.field(i, f), o.field(f)
            assert rel_err(a, b, field_floor(f, b)) <= 1e-8, (i, f)


@pytest.mark.gpu
def test_ensemble_equals_single_problem_path(gpu_lib):
    """Instance i of the ensemble and a single-problem handle with the same
    parameters step through bit-identical states."""
    ens = gpu_lib.Ensemble(SMALL)
    init = [ens.scalars(i) for i in range(len(SMALL))]
    ens.run(40)
    for i, spec in enumerate(SMALL):
        g = gpu_lib.Domain(gpu_lib.LuleshProblem(nx=spec["nx"], nr=spec["nr"]))
        g.hgcoef = spec["hgcoef"]
        if spec["einit"] > 0:
            e = g.field("e")
            e[0] = spec["einit"]
            g.set_field("e", e)
        g.deltatime = init[i]["deltatime"]
        gpu_lib.run(g, 40)
        for f in STATE:
            assert np.array_equal(ens.field(i, f), g.field(f)), (i, f)
        assert ens.scalars(i)["time"] == g.time


@pytest.mark.gpu
def test_reset_and_tuning_do_not_change_results(gpu_lib):
    ens = gpu_lib.Ensemble(SMALL)
    ens.run(25)
    first = [ens.field(i, "e") for i in range(len(SMALL))]
    chosen = ens.autotune(cycles=2)
    assert chosen["force_block"] in (64, 128, 256) and chosen["node_block"] in (128, 256, 512)
    assert all(ens.scalars(i)["cycle"] == 0 for i in range(len(SMALL)))  # back to the start
    ens.set_tuning(force_block=64, kin_block=256, mat_block=64, node_block=512)
    ens.run(25)
    for i in range(len(SMALL)):
        assert np.array_equal(ens.field(i, "e"), first[i]), i
    ens.reset()
    assert ens.scalars(0)["cycle"] == 0 and ens.scalars(0)["time"] == 0.0


@pytest.mark.gpu
def test_single_problem_autotune_keeps_state(gpu_lib):
    g = gpu_lib.Domain(gpu_lib.LuleshProblem(nx=20))
    gpu_lib.run(g, 10)
    before = {f: g.field(f) for f in ("e", "xd")}
    t0, c0 = g.time, g.cycle
    g.autotune(cycles=2)
    assert g.time == t0 and g.cycle == c0
    for f, v in before.items():
        assert np.array_equal(g.field(f), v), f


@pytest.mark.gpu
def test_ensemble_stops_each_instance_at_stoptime(gpu_lib):
    ens = gpu_lib.Ensemble([{"nx": 4}, {"nx": 6, "hgcoef": 2.5}], mode=7)
    ens.run(10**9)
    for i in range(2):
        s = ens.scalars(i)
        assert s["time"] == 1e-2 and s["status"] == 0, (i, s)


def c4_sample(instances, k=16, seed=0xC4):
    """A seeded sample of k instance indices of the C4 draw that always holds
    the smallest and the largest mesh and both region counts."""
    nxs = [s["nx"] for s in instances]
    must = {int(np.argmin(nxs)), int(np.argmax(nxs))}
    must.add(next(i for i, s in enumerate(instances) if s["nr"] == 1))
    must.add(next(i for i, s in enumerate(instances) if s["nr"] == 11))
    rest = [i for i in range(len(instances)) if i not in must]
    rng = np.random.default_rng(seed)
    pick = rng.choice(rest, size=k - len(must), replace=False)
    return sorted(must | {int(i) for i in pick})


@pytest.mark.gpu
def test_c4_draw_matches_oracle(gpu_lib, oracle_mod):
    """The batched-ensemble configuration itself: the 256-instance draw of
    seed 0xC4 (nx uniform in [16, 64], energy factor in [0.5, 2], hgcoef in
    [2, 4], 1 or 11 regions) advanced 300 cycles as one ensemble; a seeded
    sample of 16 instances, holding the smallest and largest meshes and both
    region counts, is compared with the oracle run of the same instance."""
    draw = gpu_lib.sedov_instances(0xC4, 256, 16, 64)
    ens = gpu_lib.Ensemble(draw, mode=0)
    iters = 300
    ens.run(iters)
    sample = c4_sample(draw)
    assert len(sample) == 16
    assert {draw[i]["nr"] for i in sample} == {1, 11}
    assert min(draw[i]["nx"] for i in sample) == min(s["nx"] for s in draw)
    assert max(draw[i]["nx"] for i in sample) == max(s["nx"] for s in draw)
    for i in sample:
        spec = draw[i]
        o = oracle_mod.OracleDomain(spec["nx"], nr=spec["nr"], mode=0, seed=spec["region_seed"])
        o.set("hgcoef", spec["hgcoef"])
        o.set_einit(spec["einit"])
        assert o.run(iters) == 0
        s = ens.scalars(i)
        assert s["status"] == 0, i
        assert s["cycle"] == o.get("cycle"), i
        assert s["cycle"] == iters or o.get("time") >= o.get("stoptime"), i
        assert s["time"] == pytest.approx(o.get("time"), rel=1e-12), i
        assert s["dtcourant"] == pytest.approx(o.get("dtcourant"), rel=1e-12), i
        assert ens.field(i, "e")[0] == pytest.approx(o.field("e")[0], rel=1e-9), i
        for f in STATE + ["vdov", "arealg"]:
            a, b = ens.field(i, f), o.field(f)
            assert rel_err(a, b, field_floor(f, b)) <= 1e-8, (i, f)
        o.close()
    ens.close()


@pytest.mark.gpu
def test_single_instance_ensemble_is_the_single_problem(gpu_lib):
    spec = {"nx": 10, "nr": 11, "hgcoef": 2.7, "einit": 1.3 * 3.948746e7 * (10 / 45) ** 3}
    ens = gpu_lib.Ensemble([spec])
    dt0 = ens.scalars(0)["deltatime"]
    ens.run(50)
    g = gpu_lib.Domain(gpu_lib.LuleshProblem(nx=10, nr=11))
    g.hgcoef = spec["hgcoef"]
    e = g.field("e")
    e[0] = spec["einit"]
    g.set_field("e", e)
    g.deltatime = dt0
    gpu_lib.run(g, 50)
    for f in STATE:
        assert np.array_equal(ens.field(0, f), g.field(f)), f
    assert ens.scalars(0)["time"] == g.time
