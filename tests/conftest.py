import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "lulesh.jl_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built liblulesh_gb300.so")


def rel_err(a, b, floor):
    """max |a-b| / max(|b|, floor), the per-field parity metric."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.size == 0:
        return 0.0
    den = np.maximum(np.abs(b), floor)
    return float(np.max(np.abs(a - b) / den))


# Per-field floors for the relative-error metric: a field's cut-off (values
# below it are snapped to zero by the method) or 1e-12 of its largest value.
# delv = vnew - v is a difference of relative volumes of order 1, so one ulp
# of its operands (~2e-16) is its accuracy: its floor is 1e-7 (1e-15 absolute
# at the 1e-8 bar).
CUTS = {"e": 1e-7, "p": 1e-7, "q": 1e-7, "xd": 1e-7, "yd": 1e-7, "zd": 1e-7, "v": 1e-10,
        "delv": 1e-7}


def field_floor(name, ref):
    m = float(np.max(np.abs(ref))) if np.size(ref) else 0.0
    return max(CUTS.get(name, 0.0), 1e-12 * m, 1e-300)


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    """The product library, built in-tree; skips nothing: a missing GPU fails."""
    import lulesh_gb300
    if not os.path.exists(lulesh_gb300.library_path()):
        import build_gb300
        build_gb300.build()
    return lulesh_gb300
