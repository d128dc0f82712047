"""GPU parity of liblulesh_gb300 against the CPU oracle (through the C ABI).

Tolerances (the FP64 parity bar): the same cycle count and final time
(relative 1e-12), origin energy to relative 1e-9 and every field to a maximum
relative error of 1e-8, with the field's cut-off (or 1e-12 of its largest
magnitude) as the floor of the denominator. Integer and setup fields must be
bit-identical.
"""
import json
import os

import numpy as np
import pytest

from conftest import ROOT, field_floor, rel_err

pytestmark = pytest.mark.gpu

FIELD_TOL = 1e-8
STATE_F64 = ["e", "p", "q", "v", "ss", "x", "y", "z", "xd", "yd", "zd"]
STEP_F64 = STATE_F64 + ["vnew", "delv", "arealg", "vdov", "delv_xi", "delv_eta", "delv_zeta",
                        "delx_xi", "delx_eta", "delx_zeta"]
AUX_F64 = ["fx", "fy", "fz", "xdd", "ydd", "zdd", "dxx", "dyy", "dzz", "ql", "qq"]
INDEX_FIELDS = ["nodelist", "lxim", "lxip", "letam", "letap", "lzetam", "lzetap", "symmX", "symmY",
                "symmZ", "nodeElemCount", "nodeElemStart", "nodeElemCornerList", "matElemlist",
                "regNumList", "regElemlist", "regCSR", "regReps", "regSorted", "regElemSize"]


def pair(L, oracle_mod, nx, mode=0, nr=11, keep_aux=False, balance=1, cost=1):
    g = L.Domain(L.LuleshProblem(nx=nx, nr=nr, mode=mode, keep_aux=keep_aux, balance=balance, cost=cost))
    o = oracle_mod.OracleDomain(nx, nr=nr, mode=mode, balance=balance, cost=cost)
    return g, o


# The kept auxiliary fields are nodal sums with heavy cancellation (forces,
# accelerations) or deviatoric differences; their floor is 1e-7 of the
# field's largest magnitude.
AUX_FLOOR = 1e-7


def assert_fields(g, o, names, tol=FIELD_TOL, where=""):
    worst = {}
    for n in names:
        a, b = g.field(n), o.field(n)
        assert a.shape == b.shape, n
        floor = field_floor(n, b)
        if n in AUX_F64:
            floor = max(floor, AUX_FLOOR * float(np.max(np.abs(b))))
        worst[n] = rel_err(a, b, floor)
    bad = {k: v for k, v in worst.items() if not (v <= tol)}
    assert not bad, f"{where} fields beyond {tol}: {bad}"
    return worst


def assert_scalars(g, o, rel=1e-12):
    for s in ["time", "deltatime", "dtcourant", "dthydro"]:
        assert getattr(g, s) == pytest.approx(o.get(s), rel=rel), s
    assert g.cycle == o.get("cycle")


def test_setup_is_bit_identical(gpu_lib, oracle_mod):
    g, o = pair(gpu_lib, oracle_mod, 7, nr=11, balance=2, cost=3)
    for n in INDEX_FIELDS:
        assert np.array_equal(g.field(n), o.field(n)), n
    assert np.array_equal(g.field("elemBC"), o.field("elemBC"))
    for n in ["x", "y", "z", "volo", "elemMass", "nodalMass", "e", "v", "p", "q", "ss", "xd"]:
        assert np.array_equal(g.field(n), o.field(n)), n
    assert g.deltatime == o.get("deltatime")
    for s in gpu_lib.SCALARS:
        if s != "cycle":
            assert getattr(g, s) == o.get(s), s


@pytest.mark.parametrize("mode", [0, 1, 2, 4, 7])
def test_first_steps_match(gpu_lib, oracle_mod, mode):
    g, o = pair(gpu_lib, oracle_mod, 6, mode=mode, keep_aux=True)
    for step in range(4):
        gpu_lib.timeIncrement(g)
        o.time_increment()
        gpu_lib.lagrangeLeapFrog(g)
        assert o.lagrange_leapfrog() == 0
        assert_scalars(g, o)
        assert_fields(g, o, STATE_F64, tol=1e-10, where=f"step {step}")
        assert_fields(g, o, STEP_F64 + AUX_F64, where=f"step {step}")


@pytest.mark.parametrize("nx,seed", [(6, s) for s in range(6)] + [(12, 100), (12, 101)])
@pytest.mark.parametrize("mode", [0, 1, 2, 4, 7])
def test_random_states_match_oracle(gpu_lib, oracle_mod, mode, nx, seed):
    """Seeded random states on 6^3 and 12^3 meshes (energies, pressures, viscosities,
    sound speeds, relative volumes within 3 % of 1, velocities with exact
    zeros, a random hourglass coefficient) stepped three cycles with every
    step and auxiliary field compared: the limiter's cases, the clamps, the
    cut-offs and the EOS branches that the Sedov blast reaches rarely or late."""
    rng = np.random.default_rng(seed)
    g, o = pair(gpu_lib, oracle_mod, nx, mode=mode, keep_aux=True)
    E, N = g.numElem, g.numNode
    state = {"e": rng.uniform(0, 2e4, E) * (rng.random(E) < 0.7),
             "p": rng.uniform(0, 1e3, E) * (rng.random(E) < 0.5),
             "q": rng.uniform(0, 50, E) * (rng.random(E) < 0.3),
             "v": rng.uniform(0.97, 1.03, E), "ss": rng.uniform(0, 50, E)}
    for f in ("xd", "yd", "zd"):
        state[f] = rng.normal(0, 0.5, N) * (rng.random(N) < 0.6)
    for f, v in state.items():
        g.set_field(f, v)
        o.set_field(f, v)
    hg = float(rng.uniform(1, 4))
    g.hgcoef = hg
    o.set("hgcoef", hg)
    for step in range(3):
        gpu_lib.timeIncrement(g)
        o.time_increment()
        gpu_lib.lagrangeLeapFrog(g)
        assert o.lagrange_leapfrog() == 0
        assert_scalars(g, o)
        assert_fields(g, o, STEP_F64 + AUX_F64, where=f"step {step}")


# The limiter's face masks (interior 0, then symmetry, free and comm bits of
# each face's three), src/types.jl's XI_M .. ZETA_P_COMM
FACE_BITS = [(0x1, 0x2, 0x4), (0x8, 0x10, 0x20), (0x40, 0x80, 0x100),
             (0x200, 0x400, 0x800), (0x1000, 0x2000, 0x4000), (0x8000, 0x10000, 0x20000)]
NEIGHBOURS = ["lxim", "lxip", "letam", "letap", "lzetam", "lzetap"]


@pytest.mark.parametrize("mode,seed", [(0, 0xBC0), (1, 0xBC1), (4, 0xBC2), (7, 0xBC3)])
def test_random_boundary_masks_and_neighbours_match_oracle(gpu_lib, oracle_mod, mode, seed):
    """Every face of every element takes a random limiter case (interior,
    symmetry, free or comm; src/domain.jl:2330-2420) and a random neighbour
    element, on a random state: the GPU's neighbour reads, the faithful
    xi-plus offset included, are the oracle's in every case. A single-rank
    Sedov mesh has no comm faces and symmetry or free faces only on its six
    boundary planes."""
    rng = np.random.default_rng(seed)
    g, o = pair(gpu_lib, oracle_mod, 6, mode=mode, keep_aux=True)
    E, N = g.numElem, g.numNode
    state = {"e": rng.uniform(0, 2e4, E), "p": rng.uniform(0, 1e3, E) * (rng.random(E) < 0.5),
             "q": rng.uniform(0, 50, E) * (rng.random(E) < 0.3), "v": rng.uniform(0.97, 1.03, E),
             "ss": rng.uniform(0, 50, E)}
    for f in ("xd", "yd", "zd"):
        state[f] = rng.normal(0, 0.5, N)
    bc = np.zeros(E, np.uint32)
    for bits in FACE_BITS:
        bc |= np.array((0,) + bits, np.uint32)[rng.integers(0, 4, E)]
    state["elemBC"] = bc
    for name in NEIGHBOURS:
        # the faithful xi-plus read is element lxip - 1, so lxip >= 1 there
        lo = 1 if (name == "lxip" and not mode & 4) else 0
        state[name] = rng.integers(lo, E, E).astype(np.int64)
    for f, v in state.items():
        g.set_field(f, v)
        o.set_field(f, v)
    for n in ["elemBC"] + NEIGHBOURS:
        assert np.array_equal(g.field(n), o.field(n)), n
    for step in range(3):
        gpu_lib.timeIncrement(g)
        o.time_increment()
        gpu_lib.lagrangeLeapFrog(g)
        assert o.lagrange_leapfrog() == 0
        assert_scalars(g, o)
        assert_fields(g, o, STEP_F64 + AUX_F64, where=f"step {step}")


@pytest.mark.parametrize("mode", [0, 7])
def test_one_step_from_developed_state(gpu_lib, oracle_mod, mode):
    """Load the oracle's state after 120 cycles into the GPU and take one step."""
    nx = 12
    g, o = pair(gpu_lib, oracle_mod, nx, mode=mode, keep_aux=True)
    assert o.run(120) == 0
    for n in STATE_F64:
        g.set_field(n, o.field(n))
    for s in ["time", "deltatime", "dtcourant", "dthydro", "cycle"]:
        setattr(g, s, o.get(s))
    gpu_lib.timeIncrement(g)
    o.time_increment()
    gpu_lib.lagrangeLeapFrog(g)
    assert o.lagrange_leapfrog() == 0
    assert_scalars(g, o)
    assert_fields(g, o, STATE_F64, tol=1e-10)
    assert_fields(g, o, STEP_F64 + AUX_F64)


GOLDEN = json.load(open(os.path.join(ROOT, "tests", "golden", "oracle_runs.json")))


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_run_parity(gpu_lib, oracle_mod, name):
    c = GOLDEN[name]
    g, o = pair(gpu_lib, oracle_mod, c["nx"], mode=c["mode"])
    s = gpu_lib.run(g, c["num_iters"])
    assert o.run(c["num_iters"]) == 0
    assert s["cycle"] == o.get("cycle") == c["cycle"]
    assert s["time"] == pytest.approx(o.get("time"), rel=1e-12)
    assert g.field("e")[0] == pytest.approx(o.field("e")[0], rel=1e-9)
    assert_fields(g, o, STATE_F64 + ["arealg", "vdov", "delv"])
    # LULESH's own symmetry check gives the same numbers
    e0, maxabs, total, maxrel = gpu_lib.verify(g)
    omaxabs, ototal, omaxrel = o.symmetry()
    scale = np.abs(o.field("e")[: c["nx"] ** 2]).max()
    assert abs(maxabs - omaxabs) <= 1e-8 * scale
    assert abs(total - ototal) <= 1e-8 * scale * c["nx"] ** 2


def test_reference_default_run_matches_oracle(gpu_lib, oracle_mod):
    """examples/benchmark.jl with its defaults (src/utils.jl:13-20: N = 45,
    num_iters = 10; examples/benchmark.jl:23-26: one region, balance and
    cost 1), through the per-step calls in the loop of
    examples/benchmark.jl:82-98."""
    L = gpu_lib
    g, o = pair(L, oracle_mod, 45, nr=1)
    while g.time < g.stoptime:
        L.timeIncrement(g)
        L.lagrangeLeapFrog(g)
        if g.cycle >= 10:
            break
    assert o.run(10) == 0
    assert g.cycle == o.get("cycle") == 10
    assert_scalars(g, o)
    assert g.field("e")[0] == pytest.approx(o.field("e")[0], rel=1e-9)
    assert_fields(g, o, STATE_F64 + ["arealg", "vdov", "delv"])


def test_run_equals_stepwise_and_is_deterministic(gpu_lib, oracle_mod):
    a = gpu_lib.Domain(gpu_lib.LuleshProblem(nx=10))
    b = gpu_lib.Domain(gpu_lib.LuleshProblem(nx=10))
    c = gpu_lib.Domain(gpu_lib.LuleshProblem(nx=10))
    gpu_lib.run(a, 75)
    gpu_lib.run(c, 75)
    for _ in range(75):
        gpu_lib.timeIncrement(b)
        gpu_lib.lagrangeLeapFrog(b)
    for n in STATE_F64 + ["vdov", "arealg"]:
        assert np.array_equal(a.field(n), b.field(n)), n
        assert np.array_equal(a.field(n), c.field(n)), n
    assert a.time == b.time and a.dtcourant == b.dtcourant and a.cycle == b.cycle == 75


def test_run_to_stoptime_stops_exactly(gpu_lib):
    g = gpu_lib.Domain(gpu_lib.LuleshProblem(nx=10, mode=gpu_lib.MODE_LULESH2))
    s = gpu_lib.run(g, 10**9)
    assert s["time"] == 1e-2
    s2 = gpu_lib.run(g, 10**9)  # time >= stoptime: the loop does not enter
    assert s2["cycle"] == s["cycle"]


def test_num_iters_semantics(gpu_lib):
    g = gpu_lib.Domain(gpu_lib.LuleshProblem(nx=6))
    assert gpu_lib.run(g, 5)["cycle"] == 5
    assert gpu_lib.run(g, 5)["cycle"] == 6   # benchmark.jl always takes one step
    assert gpu_lib.run(g, 40)["cycle"] == 40


# ---- errors: the reference's error(...) sites, provoked on the host ----------

def test_qstop_error(gpu_lib, oracle_mod):
    g, o = pair(gpu_lib, oracle_mod, 6)
    gpu_lib.run(g, 10)
    o.run(10)
    assert o.field("q").max() > 0.0
    g.qstop = 1e-30
    o.set("qstop", 1e-30)
    gpu_lib.timeIncrement(g)
    o.time_increment()
    with pytest.raises(gpu_lib.LuleshError, match="QStopError"):
        gpu_lib.lagrangeLeapFrog(g)
    assert o.lagrange_leapfrog() == 2


def test_inverted_element_volume_error(gpu_lib, oracle_mod):
    g, o = pair(gpu_lib, oracle_mod, 4)
    x = g.field("x")
    x[1] = -0.9  # drag a node of element 0 through its neighbour
    g.set_field("x", x)
    o.view("x")[1] = -0.9
    gpu_lib.timeIncrement(g)
    o.time_increment()
    with pytest.raises(gpu_lib.LuleshError, match="Early Volume Error"):
        gpu_lib.lagrangeLeapFrog(g)
    assert o.lagrange_leapfrog() == 1 and o.error_site() == 1


def test_negative_relative_volume_error(gpu_lib, oracle_mod):
    g, o = pair(gpu_lib, oracle_mod, 4)
    v = g.field("v")
    v[5] = -1.0
    g.set_field("v", v)
    o.view("v")[5] = -1.0
    gpu_lib.timeIncrement(g)
    o.time_increment()
    with pytest.raises(gpu_lib.LuleshError, match="Volume Error: Volume is negative"):
        gpu_lib.lagrangeLeapFrog(g)
    assert o.lagrange_leapfrog() == 1 and o.error_site() == 2


def test_bad_bc_mask_error(gpu_lib, oracle_mod):
    g, o = pair(gpu_lib, oracle_mod, 4)
    bc = g.field("elemBC")
    bc[0] |= 0x2  # XI_M_SYMM | XI_M_FREE is not a valid case
    g.set_field("elemBC", bc)
    o.view("elemBC")[0] |= 0x2
    gpu_lib.timeIncrement(g)
    o.time_increment()
    with pytest.raises(gpu_lib.LuleshError, match="^Error$"):
        gpu_lib.lagrangeLeapFrog(g)
    assert o.lagrange_leapfrog() == 3


@pytest.mark.parametrize("path", ["stepwise", "device_run"])
def test_courant_constraint_not_registered_at_or_above_1e20(gpu_lib, oracle_mod, path):
    """calcCourantConstraintForElems starts its minimum at 1.0e+20 and keeps a
    candidate only if it is strictly below (src/domain.jl:2966, 3003-3014):
    when every active element's arealg/sqrt(dtf) is >= 1e20, dtcourant keeps
    its old value. Provoked on the host: a 2^3 mesh scaled by 200 (elements
    of edge 112.5, relative volume 8e6 after the step), a cold state (e = p =
    q = 0, so ss takes its 3.3e-19 floor) and a uniform expansion (every
    element active, vdov > 0)."""
    L = gpu_lib
    g, o = pair(L, oracle_mod, 2, mode=0)
    for n in ["x", "y", "z"]:
        pos = o.field(n) * 200.0
        g.set_field(n, pos)
        o.set_field(n, pos)
        vel = 1e-3 * pos
        g.set_field(n + "d", vel)
        o.set_field(n + "d", vel)
    zero = np.zeros(8)
    for n in ["e", "p", "q"]:
        g.set_field(n, zero)
        o.set_field(n, zero)
    g.dtcourant = 0.5
    o.set("dtcourant", 0.5)
    if path == "stepwise":
        L.timeIncrement(g)
        L.lagrangeLeapFrog(g)
    else:
        L.run(g, 1)
    o.time_increment()
    assert o.lagrange_leapfrog() == 0
    # the precondition: every element active, every Courant candidate >= 1e20
    vdov, arealg, ss = o.field("vdov"), o.field("arealg"), o.field("ss")
    assert np.all(vdov > 0.0)
    assert np.all(arealg / ss >= 1e20)
    assert o.get("dtcourant") == 0.5
    assert g.dtcourant == 0.5
    assert g.dthydro == pytest.approx(o.get("dthydro"), rel=1e-12)
    assert g.dthydro < 1e20
    assert_scalars(g, o)
    assert_fields(g, o, STATE_F64 + ["vdov", "arealg"])
    # the next cycle's timeIncrement! sees the kept value in both
    L.timeIncrement(g)
    o.time_increment()
    assert g.deltatime == pytest.approx(o.get("deltatime"), rel=1e-12)


def test_error_stops_device_run(gpu_lib):
    g = gpu_lib.Domain(gpu_lib.LuleshProblem(nx=6))
    gpu_lib.run(g, 10)
    assert g.field("q").max() > 0.0
    g.qstop = 1e-30
    with pytest.raises(gpu_lib.LuleshError, match="QStopError"):
        gpu_lib.run(g, 50)
    assert g.cycle == 11  # the failing cycle's timeIncrement ran, nothing after


# ---- smallest meshes: every element on the boundary ------------------------------

@pytest.mark.parametrize("nx", [1, 2, 3])
@pytest.mark.parametrize("mode", [0, 7])
def test_tiny_meshes_match_oracle(gpu_lib, oracle_mod, nx, mode):
    """nx = 1 (one element, eight nodes, every face on a symmetry plane or free
    surface) to 3, stepwise to stoptime with the auxiliary fields."""
    g, o = pair(gpu_lib, oracle_mod, nx, mode=mode, keep_aux=True)
    steps = 0
    while o.get("time") < o.get("stoptime") and steps < 100:
        gpu_lib.timeIncrement(g)
        o.time_increment()
        gpu_lib.lagrangeLeapFrog(g)
        assert o.lagrange_leapfrog() == 0
        assert_scalars(g, o)
        assert_fields(g, o, STATE_F64, tol=1e-10, where=f"step {steps}")
        assert_fields(g, o, STEP_F64 + AUX_F64, where=f"step {steps}")
        steps += 1
    assert o.get("time") >= o.get("stoptime") and g.time == pytest.approx(o.get("time"), rel=1e-12)


# ---- full-size checks -----------------------------------------------------------

@pytest.mark.parametrize("mode", [0, 7])
def test_full_size_s150_matches_oracle(gpu_lib, oracle_mod, mode):
    """The benchmark problem at its stated length: 150^3 (3,375,000
    elements), 11 regions, 200 cycles, in the faithful mode and with the
    reference's defects corrected, against the oracle (OpenMP, ~25 s on 16
    host cores). Same cycle count and time, origin energy to 1e-9, every
    state field plus vdov and arealg to 1e-8, and LULESH's symmetry numbers."""
    g, o = pair(gpu_lib, oracle_mod, 150, mode=mode)
    s = gpu_lib.run(g, 200)
    assert o.run(200) == 0
    assert s["cycle"] == o.get("cycle") == 200
    assert_scalars(g, o)
    assert g.field("e")[0] == pytest.approx(o.field("e")[0], rel=1e-9)
    assert_fields(g, o, STATE_F64 + ["vdov", "arealg", "delv"])
    e0, maxabs, total, maxrel = gpu_lib.verify(g)
    omaxabs, ototal, omaxrel = o.symmetry()
    scale = np.abs(o.field("e")[: 150 ** 2]).max()
    assert abs(maxabs - omaxabs) <= 1e-8 * scale
    g.close()
    o.close()


def test_full_size_s150_is_deterministic(gpu_lib):
    a = gpu_lib.Domain(gpu_lib.LuleshProblem(nx=150))
    b = gpu_lib.Domain(gpu_lib.LuleshProblem(nx=150))
    gpu_lib.run(a, 6)
    gpu_lib.run(b, 6)
    for n in ["e", "xd", "q", "ss"]:
        assert np.array_equal(a.field(n), b.field(n)), n
    a.close()
    b.close()


C3_CYCLES = int(os.environ.get("LULESH_C3_CYCLES", "500"))


def test_largest_configuration_matches_oracle(gpu_lib, oracle_mod):
    """The unbalanced-regions problem at its full size and length (256^3 =
    16.8 M elements, 11 regions, balance 4, cost 2, 500 cycles), with the
    region cost model on in the GPU run (results unchanged by it), against
    the oracle (OpenMP, about five minutes on 16 host cores)."""
    L = gpu_lib
    g = L.Domain(L.LuleshProblem(nx=256, nr=11, balance=4, cost=2, region_reps=True))
    o = oracle_mod.OracleDomain(256, nr=11, balance=4, cost=2)
    for n in ["regNumList", "regElemSize", "regReps"]:
        assert np.array_equal(g.field(n), o.field(n)), n
    s = L.run(g, C3_CYCLES)
    assert o.run(C3_CYCLES) == 0
    assert s["cycle"] == o.get("cycle") == C3_CYCLES
    assert_scalars(g, o)
    assert g.field("e")[0] == pytest.approx(o.field("e")[0], rel=1e-9)
    assert_fields(g, o, STATE_F64 + ["vdov", "arealg", "delv"])
    g.close()
    o.close()
