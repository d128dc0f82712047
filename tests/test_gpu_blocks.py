"""The multi-rank decomposition as blocks of one mesh on one GPU
(lulesh_create_blocks): tp^3 blocks of nx^3 elements with halo copies
across the block faces give bitwise the single-block run of the whole
(tp*nx)^3 mesh, in the reference's faithful mode and with its defects
corrected, through the device run loop and the per-step calls."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE = ["e", "p", "q", "v", "ss", "x", "y", "z", "xd", "yd", "zd"]
STEP = ["vdov", "arealg", "delv", "vnew", "delv_xi", "delv_eta", "delv_zeta", "delx_xi", "delx_eta", "delx_zeta"]
NODE = {"x", "y", "z", "xd", "yd", "zd", "fx", "fy", "fz", "xdd", "ydd", "zdd", "nodalMass"}


def pair(L, nx, tp, mode, keep_aux=False):
    whole = L.Domain(L.LuleshProblem(nx=nx * tp, mode=mode, keep_aux=keep_aux))
    blocks = L.Domain(L.LuleshProblem(nx=nx, mode=mode, keep_aux=keep_aux, blocks_per_edge=tp))
    return whole, blocks


def assert_same(whole, blocks, names):
    _, eg, ng = blocks.block_map()
    for f in names:
        a, v = whole.field(f), blocks.field(f)
        ids = ng if f in NODE else eg
        # every packed copy holds the whole mesh's bits (shared nodes included)
        assert np.array_equal(v.view(np.uint64), a[ids].view(np.uint64)), f
    for s in ["time", "deltatime", "dtcourant", "dthydro", "cycle"]:
        assert getattr(whole, s) == getattr(blocks, s), s


@pytest.mark.parametrize("nx,tp,mode", [(6, 2, 0), (6, 2, 7), (4, 3, 0), (4, 3, 1), (5, 3, 4)])
def test_blocks_run_is_the_single_block_run(gpu_lib, nx, tp, mode):
    L = gpu_lib
    whole, blocks = pair(L, nx, tp, mode)
    assert blocks.numElem == whole.numElem and blocks.numNode == tp ** 3 * (nx + 1) ** 3
    # the setup: masses, volumes, positions of every copy
    assert_same(whole, blocks, ["x", "y", "z", "nodalMass", "volo", "elemMass", "e"])
    sw, sb = L.run(whole, 80), L.run(blocks, 80)
    assert sw["cycle"] == sb["cycle"] == 80
    assert_same(whole, blocks, STATE + STEP)


@pytest.mark.parametrize("mode", [0, 7])
def test_blocks_stepwise_with_aux_fields(gpu_lib, mode):
    """The per-step calls (timeIncrement!, lagrangeLeapFrog) with the kept
    auxiliary fields, from a developed state."""
    L = gpu_lib
    whole, blocks = pair(L, 4, 2, mode, keep_aux=True)
    L.run(whole, 40)
    L.run(blocks, 40)
    for _ in range(5):
        L.timeIncrement(whole)
        L.lagrangeLeapFrog(whole)
        L.timeIncrement(blocks)
        L.lagrangeLeapFrog(blocks)
    assert_same(whole, blocks, STATE + STEP + ["fx", "fy", "fz", "xdd", "ydd", "zdd", "dxx", "dyy", "dzz", "ql", "qq"])


def test_blocks_run_to_stoptime(gpu_lib):
    L = gpu_lib
    whole, blocks = pair(L, 5, 2, L.MODE_LULESH2)
    sw, sb = L.run(whole, 10 ** 9), L.run(blocks, 10 ** 9)
    assert sw["time"] == sb["time"] == 1e-2 and sw["cycle"] == sb["cycle"]
    assert_same(whole, blocks, STATE)
    # the reference's rank-0 report: origin energy and plane-0 symmetry of block 0
    e0 = L.verify(blocks)[0]
    assert e0 == whole.field("e")[0]


def test_blocks_with_the_inline_geometry_split(gpu_lib):
    L = gpu_lib
    whole, blocks = pair(L, 4, 2, 0)
    blocks.set_tuning(geometry=1)
    L.run(whole, 50)
    L.run(blocks, 50)
    assert_same(whole, blocks, STATE)


def test_blocks_errors_and_limits(gpu_lib):
    L = gpu_lib
    _, blocks = pair(L, 3, 2, 0)
    with pytest.raises(L.LuleshError):
        L.Adjoint(blocks)  # the adjoint kernels have no halo transposes
    # an error in one block stops every block: a QStop provoked on the host
    L.run(blocks, 10)
    blocks.qstop = 1e-30
    with pytest.raises(L.LuleshError, match="QStopError"):
        L.run(blocks, 20)


def test_one_block_is_the_plain_domain(gpu_lib):
    L = gpu_lib
    a = L.Domain(L.LuleshProblem(nx=7))
    b = L.Domain(L.LuleshProblem(nx=7, blocks_per_edge=1))
    L.run(a, 40)
    L.run(b, 40)
    for f in STATE + ["vdov", "arealg"]:
        assert np.array_equal(a.field(f), b.field(f)), f


def test_blocks_state_file_resumes_bitwise(gpu_lib, tmp_path):
    L = gpu_lib
    _, blocks = pair(L, 4, 2, 0)
    L.run(blocks, 20)
    path = str(tmp_path / "blocks.state")
    blocks.save_state(path)
    L.run(blocks, 45)
    after = {f: blocks.field(f) for f in STATE}
    blocks.load_state(path)
    assert blocks.cycle == 20
    L.run(blocks, 45)
    for f in STATE:
        assert np.array_equal(blocks.field(f), after[f]), f
    # a single-block handle of the block edge does not take the packed state
    single = L.Domain(L.LuleshProblem(nx=4))
    with pytest.raises(L.LuleshError):
        single.load_state(path)


@pytest.mark.parametrize("tp,mode", [(2, 0), (3, 7)])
def test_blocks_from_a_random_state(gpu_lib, tp, mode):
    """A seeded random state (no symmetry to hide a halo slot read from the
    wrong neighbour) put into the whole mesh and, through the block map, into
    every block copy; five steps later every packed value is the whole
    mesh's bit for bit."""
    L = gpu_lib
    whole, blocks = pair(L, 4, tp, mode, keep_aux=True)
    _, eg, ng = blocks.block_map()
    rng = np.random.default_rng(0xB10C + tp)
    E, N = whole.numElem, whole.numNode
    state = {"e": rng.uniform(0, 2e4, E) * (rng.random(E) < 0.7),
             "p": rng.uniform(0, 1e3, E) * (rng.random(E) < 0.5),
             "q": rng.uniform(0, 50, E) * (rng.random(E) < 0.3),
             "v": rng.uniform(0.97, 1.03, E), "ss": rng.uniform(0, 50, E)}
    for f in ("xd", "yd", "zd"):
        state[f] = rng.normal(0, 0.5, N) * (rng.random(N) < 0.6)
    for f, v in state.items():
        whole.set_field(f, v)
        blocks.set_field(f, v[ng] if f in NODE else v[eg])
    for _ in range(5):
        L.timeIncrement(whole)
        L.lagrangeLeapFrog(whole)
        L.timeIncrement(blocks)
        L.lagrangeLeapFrog(blocks)
    assert_same(whole, blocks, STATE + STEP + ["fx", "fy", "fz", "ql", "qq"])


def test_blocks_regions_per_rank_and_cost_model(gpu_lib):
    """Each block holds the region sets of its rank (draws seeded with the
    rank, region numbers rotated by it, src/domain.jl:338-465): block 0's are
    the single-rank sets of an nx^3 mesh. The region cost model (balance 4,
    cost 2, per-region EOS repetitions in region order) runs on the block
    mesh and leaves the results bitwise those of the whole mesh without it."""
    L = gpu_lib
    nx, tp = 5, 2
    blocks = L.Domain(L.LuleshProblem(nx=nx, nr=11, balance=4, cost=2, region_reps=True, blocks_per_edge=tp))
    single = L.Domain(L.LuleshProblem(nx=nx, nr=11, balance=4, cost=2))
    Eb = nx ** 3
    reg = blocks.field("regNumList")
    assert np.array_equal(reg[:Eb], single.field("regNumList"))
    assert not np.array_equal(reg[:Eb], reg[Eb:2 * Eb])
    for n in ("regReps", "regElemSize", "regSorted"):
        assert np.array_equal(blocks.field(n), single.field(n)), n
    el = blocks.field("regElemlist")
    for b in range(tp ** 3):  # each block's index set covers its own elements
        assert np.array_equal(np.sort(el[b * Eb:(b + 1) * Eb]), np.arange(b * Eb, (b + 1) * Eb) + 1)
    whole = L.Domain(L.LuleshProblem(nx=nx * tp, nr=11, balance=4, cost=2))
    L.run(whole, 40)
    L.run(blocks, 40)
    assert_same(whole, blocks, STATE)
