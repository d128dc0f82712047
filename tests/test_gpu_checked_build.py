"""The index-checked debug build (-DLULESH_CHECK): every gather of the step
kernels (node, corner and instance indices, the region order) checks its
range and records LULESH_ERR_INDEX instead of reading outside its array.

Small cases run under it in a separate process (the library is loaded once
per process): single problems of nx = 1, 2, 3, 5, 8 in the faithful and the
corrected mode, a region-cost-model run, a three-instance ensemble and a
27-block mesh (the halo copies and ghost slots checked too). None
may report an index error, and every state field must agree with the
normal build's run of the same case (relative 1e-10 with the parity floors:
the checks do not change the arithmetic).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, field_floor, rel_err

pytestmark = pytest.mark.gpu

STATE = ["e", "p", "q", "v", "ss", "x", "y", "z", "xd", "yd", "zd"]
ENSEMBLE = [
    {"nx": 4, "nr": 11, "hgcoef": 3.0, "einit": 0.0},
    {"nx": 6, "nr": 1, "hgcoef": 2.4, "einit": 0.0},
    {"nx": 3, "nr": 11, "hgcoef": 3.5, "einit": 0.0},
]

CASES = r'''
import sys
import numpy as np
import lulesh_gb300 as L

def cases():
    out = {}
    for nx in (1, 2, 3, 5, 8):
        for mode in (0, 7):
            g = L.Domain(L.LuleshProblem(nx=nx, mode=mode))
            L.run(g, 30)  # raises LuleshError on any status, the index error included
            for f in STATE:
                out[f"p{nx}_{mode}_{f}"] = g.field(f)
            g.close()
    g = L.Domain(L.LuleshProblem(nx=6, nr=11, balance=2, cost=2, region_reps=True))
    L.run(g, 20)
    for f in STATE:
        out[f"r_{f}"] = g.field(f)
    g.close()
    ens = L.Ensemble(ENSEMBLE)
    ens.run(40)
    for i in range(len(ENSEMBLE)):
        for f in STATE:
            out[f"e{i}_{f}"] = ens.field(i, f)
    for mode in (0, 7):
        g = L.Domain(L.LuleshProblem(nx=3, mode=mode, blocks_per_edge=3))
        L.run(g, 30)
        for f in STATE:
            out[f"b{mode}_{f}"] = g.field(f)
        g.close()
    return out
'''


def _cases(L):
    ns = {"L": L, "STATE": STATE, "ENSEMBLE": ENSEMBLE, "np": np}
    exec(CASES.replace("import lulesh_gb300 as L", ""), ns)
    return ns["cases"]()


def test_checked_build_runs_small_cases_clean(gpu_lib, tmp_path):
    import build_gb300
    lib = build_gb300.build(defines=("LULESH_CHECK",), lib=str(tmp_path / "lib" / "liblulesh_gb300.so"))
    out = tmp_path / "checked.npz"
    script = (f"import sys\nsys.path.insert(0, {os.path.join(ROOT, 'lulesh.jl_gb300')!r})\n"
              f"STATE = {STATE!r}\nENSEMBLE = {ENSEMBLE!r}\n" + CASES +
              f"np.savez({str(out)!r}, **cases())\n")
    env = dict(os.environ, LULESH_GB300_LIB=lib)
    r = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    checked = np.load(out)
    normal = _cases(gpu_lib)
    assert sorted(checked.files) == sorted(normal)
    bad = {}
    for k, b in normal.items():
        f = k.split("_")[-1]
        err = rel_err(checked[k], b, field_floor(f, b))
        if not err <= 1e-10:
            bad[k] = err
    assert not bad, bad
