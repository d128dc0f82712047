"""Generates tests/golden/oracle_runs.json from the CPU oracle.

The reference ships no golden vectors (test/runtests.jl only checks that
examples/benchmark.jl exits 0) and Julia is not available to run it, so
these fixtures record the oracle's outputs. Run from the repository root:
    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle  # noqa: E402

# (name, nx, mode, num_iters): the reference CI case (-s 8, 10 iterations),
# two faithful runs, and the corrected method run to stoptime.
CASES = [
    ("ci_s8_faithful", 8, oracle.FAITHFUL, 10),
    ("s16_faithful_200", 16, oracle.FAITHFUL, 200),
    ("s30_faithful_1000", 30, oracle.FAITHFUL, 1000),
    ("s30_lulesh2_stoptime", 30, oracle.LULESH2, 10**9),
]
FIELDS = ["e", "p", "q", "v", "ss", "x", "y", "z", "xd", "yd", "zd", "arealg", "vdov", "delv"]


def summarize(d):
    out = {"cycle": d.get("cycle")}
    for s in ["time", "deltatime", "dtcourant", "dthydro"]:
        out[s] = d.get(s)
    out["symmetry"] = list(d.symmetry())
    out["origin_energy"] = float(d.view("e")[0])
    fields = {}
    for f in FIELDS:
        a = d.field(f)
        idx = np.linspace(0, a.size - 1, 7).astype(int)
        fields[f] = {"sum": float(a.sum()), "abs_sum": float(np.abs(a).sum()),
                     "max": float(a.max()), "min": float(a.min()),
                     "samples": {str(int(i)): float(a[i]) for i in idx}}
    out["fields"] = fields
    return out


def main():
    oracle.build()
    res = {}
    for name, nx, mode, iters in CASES:
        d = oracle.OracleDomain(nx, nr=11, mode=mode)
        st = d.run(iters)
        assert st == 0, (name, st)
        res[name] = {"nx": nx, "mode": mode, "num_iters": iters, **summarize(d)}
        print(name, res[name]["cycle"], res[name]["origin_energy"])
    with open(os.path.join(os.path.dirname(__file__), "oracle_runs.json"), "w") as f:
        json.dump(res, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
