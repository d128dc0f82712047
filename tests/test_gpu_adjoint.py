"""The reverse-mode adjoint (lulesh_adj_*) against the dual-number oracle and
against central finite differences of the GPU run itself.

Checks:
  * block dot products: for every (output field, input field) pair of one
    cycle, <w, J v> from the dual oracle equals <J^T w, v> from the adjoint
    (relative to sum |w||Jv|, bar 1e-10); plus the hgcoef column;
  * a 30-cycle run with checkpoints every 7 cycles (a partial last segment):
    the energy objective's gradient w.r.t. e and hgcoef against the dual
    oracle, same bar;
  * gradients independent of the checkpoint interval, the domain left at the
    final state of a plain run, loss equal to the objective of that state;
  * the three reverse-sweep plans (in turn, overlapped on two tapes,
    overlapped on one) bitwise equal, also for runs stopped at stoptime;
  * a run that takes no cycle;
  * central finite differences (step 1e-6 relative) of the GPU run on a few
    directions.
The derivative is that of the branches the run takes; the inputs are chosen so
that no cut-off sits at its threshold (a positive background energy).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE = ["x", "y", "z", "xd", "yd", "zd", "e", "p", "q", "v", "ss"]
SCAL = ["time", "deltatime", "dtcourant", "dthydro"]


def snapshot(g):
    return {f: g.field(f) for f in STATE}, {s: getattr(g, s) for s in SCAL + ["cycle", "hgcoef"]}


def restore(g, snap):
    fields, scal = snap
    for f, v in fields.items():
        g.set_field(f, v)
    for s, v in scal.items():
        setattr(g, s, v)


def dual_from(oracle_mod, snap, nx, mode):
    fields, scal = snap
    d = oracle_mod.DualDomain(nx, mode=mode)
    for f, v in fields.items():
        d.set_field(f, v, np.zeros_like(v))
    for s in SCAL + ["hgcoef"]:
        d.set(s, scal[s], 0.0)
    d.set("cycle", scal["cycle"])
    return d


def developed(L, nx, mode, cycles, seed):
    """A GPU domain with a positive background energy, run `cycles` cycles."""
    g = L.Domain(L.LuleshProblem(nx=nx, mode=mode))
    rng = np.random.default_rng(seed)
    g.e = g.e + 1e4 * (1.0 + rng.random(g.numElem))
    if cycles:
        L.run(g, cycles)
    return g


def energy_weights(nx, radius, elem_mass, nodal_mass):
    h = 1.125 / nx
    c = (np.arange(nx) + 0.5) * h
    zc, yc, xc = np.meshgrid(c, c, c, indexing="ij")
    we = np.where((xc ** 2 + yc ** 2 + zc ** 2).ravel() < radius ** 2, elem_mass, 0.0)
    p = np.arange(nx + 1) * h
    zn, yn, xn = np.meshgrid(p, p, p, indexing="ij")
    wn = np.where((xn ** 2 + yn ** 2 + zn ** 2).ravel() < radius ** 2, nodal_mass, 0.0)
    return we, wn


def close(a, b, scale, tol):
    return abs(a - b) <= tol * max(scale, 1e-300)


@pytest.mark.parametrize("mode", [0, 1, 2, 7])
def test_one_cycle_block_dot_products(gpu_lib, oracle_mod, mode):
    L = gpu_lib
    nx = 6
    g = developed(L, nx, mode, 5, 0xA1)
    snap = snapshot(g)
    rng = np.random.default_rng(0xA2)
    fields = snap[0]
    w = {f: rng.standard_normal(fields[f].size) for f in STATE}
    scale = {f: np.mean(np.abs(fields[f])) + 1e-3 for f in STATE}
    v = {f: rng.standard_normal(fields[f].size) * scale[f] for f in STATE}
    v_hg = 0.3
    # dual oracle: one run per input direction gives every output's tangent
    jv = {}
    for fi in STATE + ["hgcoef"]:
        d = dual_from(oracle_mod, snap, nx, mode)
        if fi == "hgcoef":
            d.set("hgcoef", snap[1]["hgcoef"], v_hg)
        else:
            d.set_field(fi, fields[fi], v[fi])
        assert d.cycles(1) == 0
        jv[fi] = {fo: d.field(fo)[1] for fo in STATE}
    adj = L.Adjoint(g, checkpoint_every=1)
    bad = []
    for fo in STATE:
        restore(g, snap)
        adj.clear_seeds()
        adj.set_seed(fo, w[fo])
        adj.gradient(1)
        assert adj.result.cycles == 1
        for fi in STATE + ["hgcoef"]:
            a = float(np.dot(w[fo], jv[fi][fo]))
            a_scale = float(np.dot(np.abs(w[fo]), np.abs(jv[fi][fo])))
            if fi == "hgcoef":
                b = adj.result.grad_hgcoef * v_hg
                b_scale = abs(b)
            else:
                gi = adj.grad(fi)
                b = float(np.dot(gi, v[fi]))
                b_scale = float(np.dot(np.abs(gi), np.abs(v[fi])))
            if not close(a, b, max(a_scale, b_scale), 1e-10):
                bad.append((fo, fi, a, b, max(a_scale, b_scale)))
    adj.close()
    assert not bad, bad


@pytest.mark.parametrize("mode,seed", [(0, 0xD0), (0, 0xD1), (7, 0xD2)])
def test_one_cycle_dot_products_from_random_states(gpu_lib, oracle_mod, mode, seed):
    """The block dot products of one cycle from a seeded random state
    (positive energies, random pressures, viscosities, sound speeds, relative
    volumes within 3 % of 1, velocities with exact zeros, random hourglass
    coefficient), which takes the transposes through limiter cases, clamps
    and the compression / expansion branches of the EOS that a developed
    Sedov state at one cycle does not reach."""
    L = gpu_lib
    nx = 6
    g = L.Domain(L.LuleshProblem(nx=nx, mode=mode))
    rng = np.random.default_rng(seed)
    E, N = g.numElem, g.numNode
    g.set_field("e", rng.uniform(1e2, 2e4, E))
    g.set_field("p", rng.uniform(0, 1e3, E) * (rng.random(E) < 0.5))
    g.set_field("q", rng.uniform(0, 50, E) * (rng.random(E) < 0.3))
    g.set_field("v", rng.uniform(0.97, 1.03, E))
    g.set_field("ss", rng.uniform(1, 50, E))
    for f in ("xd", "yd", "zd"):
        g.set_field(f, rng.normal(0, 0.5, N) * (rng.random(N) < 0.6))
    g.hgcoef = float(rng.uniform(1, 4))
    snap = snapshot(g)
    fields = snap[0]
    w = {f: rng.standard_normal(fields[f].size) for f in STATE}
    scale = {f: np.mean(np.abs(fields[f])) + 1e-3 for f in STATE}
    v = {f: rng.standard_normal(fields[f].size) * scale[f] for f in STATE}
    jv = {}
    for fi in STATE:
        d = dual_from(oracle_mod, snap, nx, mode)
        d.set_field(fi, fields[fi], v[fi])
        assert d.cycles(1) == 0
        jv[fi] = {fo: d.field(fo)[1] for fo in STATE}
    adj = L.Adjoint(g, checkpoint_every=1)
    bad = []
    for fo in STATE:
        restore(g, snap)
        adj.clear_seeds()
        adj.set_seed(fo, w[fo])
        adj.gradient(1)
        for fi in STATE:
            a = float(np.dot(w[fo], jv[fi][fo]))
            a_scale = float(np.dot(np.abs(w[fo]), np.abs(jv[fi][fo])))
            gi = adj.grad(fi)
            b = float(np.dot(gi, v[fi]))
            b_scale = float(np.dot(np.abs(gi), np.abs(v[fi])))
            if not close(a, b, max(a_scale, b_scale), 1e-10):
                bad.append((fo, fi, a, b, max(a_scale, b_scale)))
    adj.close()
    assert not bad, bad


@pytest.mark.parametrize("mode,hgcoef", [(0, None), (1, None), (2, None), (7, None), (0, 0.0)])
def test_run_gradient_matches_dual_oracle(gpu_lib, oracle_mod, mode, hgcoef):
    """Modes 1 and 2 take the face-5 and volume-derivative corrections one
    at a time (each changes the force transpose on its own); hgcoef 0 runs
    without hourglass forces."""
    L = gpu_lib
    nx, cycles, radius = 8, 30, 0.3
    g = developed(L, nx, mode, 0, 0xB1)
    if hgcoef is not None:
        g.hgcoef = hgcoef
    snap = snapshot(g)
    rng = np.random.default_rng(0xB2)
    de = rng.standard_normal(g.numElem) * snap[0]["e"]
    dhg = 0.2
    adj = L.Adjoint(g, radius=radius, checkpoint_every=7)
    loss = adj.gradient(cycles)
    assert adj.result.cycles == cycles and adj.result.checkpoints == 5
    ge, ghg = adj.grad("e"), adj.result.grad_hgcoef
    d = dual_from(oracle_mod, snap, nx, mode)
    d.set_field("e", snap[0]["e"], de)
    d.set("hgcoef", snap[1]["hgcoef"], dhg)
    assert d.cycles(cycles) == 0
    we, wn = energy_weights(nx, radius, d.field("elemMass")[0], d.field("nodalMass")[0])
    e, te = d.field("e")
    ref_loss = float(np.dot(we, e))
    jvp = float(np.dot(we, te))
    jscale = float(np.dot(np.abs(we), np.abs(te)))
    for c in ("xd", "yd", "zd"):
        u, tu = d.field(c)
        ref_loss += 0.5 * float(np.dot(wn, u * u))
        jvp += float(np.dot(wn, u * tu))
        jscale += float(np.dot(np.abs(wn), np.abs(u * tu)))
    assert loss == pytest.approx(ref_loss, rel=1e-10)
    vjp = float(np.dot(ge, de)) + ghg * dhg
    assert close(jvp, vjp, jscale, 1e-10), (jvp, vjp, jscale)
    adj.close()


def test_checkpoint_interval_and_final_state(gpu_lib):
    L = gpu_lib
    nx, cycles = 8, 23
    g = developed(L, nx, 0, 0, 0xC1)
    snap = snapshot(g)
    ref = L.Domain(L.LuleshProblem(nx=nx))
    restore(ref, snap)
    for _ in range(cycles):
        L.timeIncrement(ref)
        L.lagrangeLeapFrog(ref)
    grads = []
    for k in (1, 5, 23, 40):
        restore(g, snap)
        adj = L.Adjoint(g, checkpoint_every=k)
        loss = adj.gradient(cycles)
        grads.append((loss, adj.result.grad_hgcoef, {f: adj.grad(f) for f in STATE}))
        for f in STATE:
            assert np.array_equal(g.field(f), ref.field(f)), (k, f)
        for s in SCAL + ["cycle"]:
            assert getattr(g, s) == getattr(ref, s), (k, s)
        assert loss == adj.loss()
        adj.close()
    for other in grads[1:]:
        assert other[0] == grads[0][0] and other[1] == grads[0][1]
        for f in STATE:
            assert np.array_equal(other[2][f], grads[0][2][f]), f


@pytest.mark.parametrize("every,stop_early", [(7, False), (7, True), (14, False), (5, False), (5, True)])
def test_reverse_sweep_plans_agree(gpu_lib, every, stop_early):
    """The three reverse-sweep plans give bitwise the same gradients and
    final state: sequential (mode 0: one tape, the last segment taped by the
    forward sweep), overlapped on two tapes (mode 1 here: the forward sweep
    tapes the last two segments) and overlapped on one tape (mode 2:
    consecutive segments fill the tape in opposite slot orders, the
    recompute writing each slot once the transpose has released it). Cases:
    27 cycles in segments of 7 (a partial last one) and of 5 (six segments,
    partial last), runs that reach stoptime after about 17 cycles (inside the
    third of four segments, or the fourth of six), and segments of 14."""
    L = gpu_lib
    nx, cycles = 8, 27
    g = developed(L, nx, 0, 0, 0xC7)
    snap = snapshot(g)
    stoptime = g.stoptime
    if stop_early:
        ref = L.Domain(L.LuleshProblem(nx=nx))
        restore(ref, snap)
        for _ in range(17):
            L.timeIncrement(ref)
            L.lagrangeLeapFrog(ref)
        stoptime = ref.time
    out = []
    for mode in (1, 0, 2, 1, 2):
        restore(g, snap)
        g.stoptime = stoptime
        adj = L.Adjoint(g, checkpoint_every=every)
        adj.set_overlap(mode)
        loss = adj.gradient(cycles)
        if stop_early:
            assert 17 <= adj.result.cycles < cycles
        else:
            assert adj.result.cycles == cycles and adj.result.checkpoints == -(-cycles // every)
        assert adj.result.sweep == mode, (mode, adj.result.sweep)
        out.append((loss, adj.result.grad_hgcoef, {f: adj.grad(f) for f in STATE},
                    {f: g.field(f) for f in STATE}))
        adj.close()
    for other in out[1:]:
        assert other[0] == out[0][0] and other[1] == out[0][1]
        for f in STATE:
            assert np.array_equal(other[2][f], out[0][2][f]), f
            assert np.array_equal(other[3][f], out[0][3][f]), f


def test_gradient_matches_central_fd(gpu_lib):
    L = gpu_lib
    nx, cycles, h = 12, 40, 1e-6
    g = L.Domain(L.LuleshProblem(nx=nx))
    rng = np.random.default_rng(0xC5)
    e0 = g.e
    e0[1:] = rng.uniform(0.0, 1e-3, g.numElem - 1) + 1e-2
    g.e = e0
    snap = snapshot(g)
    adj = L.Adjoint(g, radius=0.3, checkpoint_every=10)
    adj.gradient(cycles)
    ge, ghg = adj.grad("e"), adj.result.grad_hgcoef
    hg0 = snap[1]["hgcoef"]

    def loss_at(e, hg):
        restore(g, snap)
        g.e = e
        g.hgcoef = hg
        L.run(g, cycles)
        assert g.cycle == cycles
        return adj.loss()

    drng = np.random.default_rng(0xF0)
    for k in range(4):
        de = drng.standard_normal(g.numElem) * e0
        dhg = (0.5 if k == 3 else 0.0) * hg0
        fd = (loss_at(e0 + h * de, hg0 + h * dhg) - loss_at(e0 - h * de, hg0 - h * dhg)) / (2 * h)
        an = float(np.dot(ge, de)) + ghg * dhg
        assert an == pytest.approx(fd, rel=2e-6, abs=1e-9 * abs(adj.result.loss)), (k, an, fd)
    adj.close()


def test_c5_gradient_matches_dual_oracle_full_size(gpu_lib, oracle_mod):
    """The 48^3, 200-cycle gradient (checkpoints every 20) of the energy
    within r < 0.3 w.r.t. e0 and hgcoef, origin energy the default and the
    others U[0, 1e-3] (seed 0xC5), against the dual-number oracle's exact JVP
    along one direction (seed 0xF0)."""
    L = gpu_lib
    nx, cycles, radius = 48, 200, 0.3
    g = L.Domain(L.LuleshProblem(nx=nx))
    rng = np.random.default_rng(0xC5)
    e0 = g.e
    e0[1:] = rng.uniform(0.0, 1e-3, g.numElem - 1)
    g.e = e0
    snap = snapshot(g)
    adj = L.Adjoint(g, radius=radius, checkpoint_every=20)
    loss = adj.gradient(cycles)
    assert adj.result.cycles == cycles and adj.result.checkpoints == 10
    ge, ghg = adj.grad("e"), adj.result.grad_hgcoef
    adj.close()
    drng = np.random.default_rng(0xF0)
    de = drng.standard_normal(g.numElem) * e0
    dhg = drng.standard_normal() * snap[1]["hgcoef"]
    d = dual_from(oracle_mod, snap, nx, 0)
    d.set_field("e", e0, de)
    d.set("hgcoef", snap[1]["hgcoef"], dhg)
    assert d.cycles(cycles) == 0
    we, wn = energy_weights(nx, radius, d.field("elemMass")[0], d.field("nodalMass")[0])
    e, te = d.field("e")
    ref_loss, jvp = float(np.dot(we, e)), float(np.dot(we, te))
    jscale = float(np.dot(np.abs(we), np.abs(te)))
    for c in ("xd", "yd", "zd"):
        u, tu = d.field(c)
        ref_loss += 0.5 * float(np.dot(wn, u * u))
        jvp += float(np.dot(wn, u * tu))
        jscale += float(np.dot(np.abs(wn), np.abs(u * tu)))
    assert loss == pytest.approx(ref_loss, rel=1e-9)
    vjp = float(np.dot(ge, de)) + ghg * dhg
    assert close(jvp, vjp, jscale, 1e-10), (jvp, vjp, jscale, abs(jvp - vjp) / jscale)


def test_gradient_of_a_run_already_at_stoptime(gpu_lib):
    """A run already at stoptime takes no cycle: its gradient is the
    objective's own (finite, zero for positions and hgcoef, the energy
    weights for e), the same for a plan of two overlapped segments and of
    one segment."""
    L = gpu_lib
    nx = 8
    g = developed(L, nx, 0, 5, 0xD1)
    g.stoptime = g.time
    snap = snapshot(g)
    out = []
    for every in (20, 40):
        restore(g, snap)
        adj = L.Adjoint(g, radius=0.3, checkpoint_every=every)
        loss = adj.gradient(40)
        assert adj.result.cycles == 0
        assert loss == adj.loss()
        grads = {f: adj.grad(f) for f in STATE}
        for f in STATE:
            assert np.all(np.isfinite(grads[f])), f
        for f in ("x", "y", "z", "p", "q", "v", "ss"):
            assert not np.any(grads[f]), f
        assert adj.result.grad_hgcoef == 0.0
        assert np.all(grads["e"] >= 0) and np.any(grads["e"])
        out.append((loss, grads))
        adj.close()
    assert out[0][0] == out[1][0]
    for f in STATE:
        assert np.array_equal(out[0][1][f], out[1][1][f]), f
