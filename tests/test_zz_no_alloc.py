"""af3d_contact_pairs_noalloc (the allocation-free contact-pair readout) against the allocating
af3d_contact_pairs, through the C ABI.  Contact-pair sets are integer data: the bar is exact set
equality, on two calls in a row for each mode.  Collected last so that it also runs after
everything else has used the device; it needs nothing from the other tests."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PAIRS = 262144


@pytest.fixture(scope="module")
def engine():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    from oracle.pyoracle import dense_state
    from tests.states import flume_system
    n = 900
    sys, fun = flume_system(n, time=0.001)
    pp = dense_state(n, 5, sys, box=(1.0, 8.0, 26.0))
    eng = af3d.Engine(sys, fun)
    eng.import_particles(pp)          # the first import derives the grid on the device
    eng.forces()
    yield eng
    eng.close()


def _noalloc(eng, cap, active):
    from avalancheflume3d_gb300._lib import lib, ptr
    out = np.full((max(cap, 1), 3), -7, dtype=np.int64)
    cnt = C.c_long(-1)
    rc = lib().af3d_contact_pairs_noalloc(eng._h, ptr(out), cap, C.byref(cnt), active)
    return rc, out, cnt.value


def _set(a):
    return set(map(tuple, np.asarray(a).tolist()))


@pytest.mark.parametrize("active", [0, 1])
def test_noalloc_pairs_equal_allocating_entry_twice(engine, active):
    want = engine.contact_pairs(active=bool(active))
    assert len(want) > 0
    for _ in range(2):
        rc, out, cnt = _noalloc(engine, MAX_PAIRS, active)
        assert rc == 0
        assert cnt == len(want)
        got = out[:cnt]
        assert len(_set(got)) == cnt and _set(got) == _set(want)


def test_noalloc_short_cap_and_limit(engine):
    from avalancheflume3d_gb300._lib import lib
    want = _set(engine.contact_pairs())
    rc, out, cnt = _noalloc(engine, 10, 0)
    assert rc == 0 and cnt == len(want) and _set(out[:10]) <= want
    rc, out, cnt = _noalloc(engine, MAX_PAIRS + 1, 0)
    assert rc == 1 and cnt == -1
    assert b"262144" in lib().af3d_last_error()


def test_noalloc_leaves_device_memory_unchanged(engine):
    import torch
    _noalloc(engine, MAX_PAIRS, 0)                 # set-up done, every kernel loaded
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for active in (0, 1, 0):
        rc, _, _ = _noalloc(engine, MAX_PAIRS, active)
        assert rc == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
