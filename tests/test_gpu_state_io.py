"""Full-state files (lulesh_save_state / lulesh_load_state): a run resumed
from a saved state matches the uninterrupted run bit for bit; the host reader
returns the saved fields; loading rejects another problem's file and a
corrupted one without touching the handle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE = ["x", "y", "z", "xd", "yd", "zd", "e", "p", "q", "v", "ss"]


@pytest.mark.parametrize("mode", [0, 7])
def test_resume_from_saved_state_is_bitwise(gpu_lib, tmp_path, mode):
    L = gpu_lib
    a = L.Domain(L.LuleshProblem(nx=12, mode=mode))
    L.run(a, 20)
    path = tmp_path / "s20.lst"
    a.save_state(str(path))
    L.run(a, 35)
    b = L.Domain(L.LuleshProblem(nx=12, mode=mode))
    b.load_state(str(path))
    assert b.cycle == 20
    L.run(b, 35)
    assert b.cycle == a.cycle == 35
    for s in ("time", "deltatime", "dtcourant", "dthydro"):
        assert getattr(a, s) == getattr(b, s), s
    for f in STATE:
        assert np.array_equal(a.field(f), b.field(f)), f


def test_reader_and_rejections(gpu_lib, tmp_path):
    L = gpu_lib
    g = L.Domain(L.LuleshProblem(nx=8))
    L.run(g, 7)
    path = tmp_path / "s7.lst"
    g.save_state(str(path))
    st = L.read_state(str(path))
    assert st["nx"] == 8 and st["numElem"] == 512 and st["scalars"]["cycle"] == 7
    for f in STATE:
        assert np.array_equal(st["fields"][f], g.field(f)), f
    other = L.Domain(L.LuleshProblem(nx=9))
    with pytest.raises(L.LuleshError):
        other.load_state(str(path))
    raw = bytearray(path.read_bytes())
    raw[200] ^= 0x40
    bad = tmp_path / "bad.lst"
    bad.write_bytes(bytes(raw))
    fresh = L.Domain(L.LuleshProblem(nx=8))
    before = fresh.field("x")
    with pytest.raises(L.LuleshError):
        fresh.load_state(str(bad))
    assert np.array_equal(fresh.field("x"), before) and fresh.cycle == 0
    with pytest.raises(ValueError):
        L.read_state(str(bad))


def test_field_download_into_caller_buffer(gpu_lib):
    """Domain.field(name, out=buf) copies into the caller's buffer (pinned
    memory in the end-to-end timing) the values field(name) returns; a buffer
    of the wrong dtype, length or layout is refused before any copy."""
    torch = pytest.importorskip("torch")
    L = gpu_lib
    g = L.Domain(L.LuleshProblem(nx=10))
    L.run(g, 5)
    for f in STATE:
        ref = g.field(f)
        buf = torch.empty(ref.size, dtype=torch.float64, pin_memory=True).numpy()
        assert g.field(f, out=buf) is buf
        assert np.array_equal(buf, ref), f
    n = g.field("e").size
    for bad in (np.empty(n, np.float32), np.empty(n - 1), np.empty((n, 2))[:, 0]):
        with pytest.raises(ValueError):
            g.field("e", out=bad)
