"""The dual-number build of the oracle (forward mode), which checks the
product's adjoint: its values must equal the double oracle's bit for bit and
its tangents must agree with central finite differences of the double oracle
on a smooth state (no cut-off or clamp near its threshold)."""
import numpy as np
import pytest

STATE = ["e", "p", "q", "v", "ss", "x", "y", "z", "xd", "yd", "zd"]


@pytest.mark.parametrize("mode", [0, 7])
def test_dual_values_equal_double_oracle(oracle_mod, mode):
    nx = 5
    o = oracle_mod.OracleDomain(nx, mode=mode, openmp=False)
    d = oracle_mod.DualDomain(nx, mode=mode)
    assert o.run(12) == 0
    assert d.cycles(12) == 0
    for f in STATE + ["delv", "vdov", "arealg", "vnew", "delv_xi", "delx_zeta"]:
        v, _ = d.field(f)
        assert np.array_equal(v, o.field(f)), f
    for s in ["time", "deltatime", "dtcourant", "dthydro"]:
        assert d.get(s)[0] == o.get(s), s


def _smooth_start(oracle_mod, nx, rng):
    """A Sedov start with a positive background energy everywhere, so that no
    pressure or energy cut-off sits at its threshold."""
    extra = 1e4 * (1.0 + rng.random(nx ** 3))
    return extra


@pytest.mark.parametrize("mode", [0, 7])
def test_dual_tangent_matches_central_fd(oracle_mod, mode):
    nx, cycles = 6, 10
    rng = np.random.default_rng(0xF0)
    extra = _smooth_start(oracle_mod, nx, rng)
    de = rng.standard_normal(nx ** 3) * 1e3
    dhg = 0.25

    def loss(eps):
        o = oracle_mod.OracleDomain(nx, mode=mode, openmp=False)
        o.set_field("e", o.field("e") + extra + eps * de)
        o.set("hgcoef", o.get("hgcoef") + eps * dhg)
        assert o.run(cycles) == 0
        u2 = o.field("xd") ** 2 + o.field("yd") ** 2 + o.field("zd") ** 2
        return float(np.sum(o.field("e") * o.field("elemMass")) + 0.5 * np.sum(o.field("nodalMass") * u2))

    d = oracle_mod.DualDomain(nx, mode=mode)
    e0, _ = d.field("e")
    d.set_field("e", e0 + extra, de)
    d.set("hgcoef", d.get("hgcoef")[0], dhg)
    assert d.cycles(cycles) == 0
    e, te = d.field("e")
    m, _ = d.field("elemMass")
    nm, _ = d.field("nodalMass")
    jvp = float(np.sum(te * m))
    for c in ("xd", "yd", "zd"):
        u, tu = d.field(c)
        jvp += float(np.sum(nm * u * tu))
    h = 1e-3
    fd = (loss(h) - loss(-h)) / (2 * h)
    assert abs(jvp - fd) <= 1e-8 * abs(fd), (jvp, fd)
