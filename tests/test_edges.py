"""Parity at the edges of the FP32 shortcuts of the force kernel, against the pinned oracle.

The search cell of every clump is estimated in FP32 and decided in FP64 only near a cell face;
the boundary routines are gated in FP32 with a slack; sphere pairs are culled in FP32 before the
exact test.  These states put clump centres on cell faces (offsets from 0 to 1e-3 of a cell, on
either side, on each axis) and spheres at grazing distance from the flume bed and side walls
(overlaps and gaps of 1e-15 to 1e-6 of the radius).  Cell indices, the sorted order and one force
pass must still be bit-identical to the oracle's.
"""
import numpy as np
import pytest

from oracle.pyoracle import PHASE_AVALANCHE, LFUNNEL, dense_state, rotate_slope, sphere_centres
from tests.states import Work, flume_system, grid_from_state, run_forces, sorted_order

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def af3d():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import avalancheflume3d_gb300 as af3d
    af3d.lib()
    return af3d


def _check(af3d, oracle, sys, fun, pp):
    n = len(pp)
    cp = grid_from_state(pp, sys, 32, oracle)
    w = Work(n, cp)
    run_forces(oracle, sys, fun, cp, pp, w, PHASE_AVALANCHE)
    ids_ref, cells_ref = sorted_order(cp, w)
    with af3d.Engine(sys, fun, ntags=32) as eng:
        eng.set_grid(cp)
        eng.import_particles(pp)
        eng.forces()
        cell_of_id, ids = eng.get_cells()
        F, T = eng.get_forces()
        contacts = eng.contact_count()
    assert np.array_equal(ids, ids_ref), "sorted (cell, id) order"
    assert np.array_equal(cell_of_id[ids_ref], cells_ref), "cell index of every clump"
    assert F.tobytes() == w.F.tobytes() and T.tobytes() == w.T.tobytes(), \
        float(np.abs(F - w.F).max())
    return cp, contacts


def test_centres_on_cell_faces(af3d, oracle):
    n = 1500
    sys, fun = flume_system(n, time=0.001)
    pp = dense_state(n, 12, sys, box=(1.0, 8.0, 26.0))
    cp = grid_from_state(pp, sys, 32, oracle)
    rng = np.random.default_rng(3)
    offsets = np.array([0.0, 1e-16, -1e-16, 1e-13, -1e-13, 1e-9, -1e-9, 2e-4, -2e-4, 1e-3, -1e-3])
    pp = pp.copy()
    r = pp["rr"].copy()
    for axis in range(3):
        pick = rng.random(n) < 0.5
        side, lo = float(cp["cell_side"][axis]), float(cp["rr_min"][axis])
        m = np.round((r[:, axis] - lo) / side)
        m = np.clip(m, 1, int(cp["ncell"][axis]) - 1)
        d = rng.choice(offsets, n)
        r[pick, axis] = lo + (m[pick] + d[pick]) * side
    pp["rr"] = r
    sphere_centres(pp)
    rotate_slope(pp, sys)
    _, contacts = _check(af3d, oracle, sys, fun, pp)
    assert contacts > 0


def test_spheres_grazing_bed_and_side_walls(af3d, oracle):
    n = 1200
    sys, fun = flume_system(n, time=0.001)
    cost, sint = float(sys["cost"]), float(sys["sint"])
    dy2, width = float(sys["dy2"]), float(sys["side"][1])
    rad = float(sys["rmax"])
    rng = np.random.default_rng(8)
    pp = dense_state(n, 19, sys, box=(1.0, 8.0, 26.0)).copy()
    # Spread the clumps along the flume in the slope frame, then move each so that its lowest
    # sphere (or its sphere nearest a side wall) sits at rad (1 + e) from that wall.
    xr = LFUNNEL + 5.0 + rng.random(n) * (float(sys["Lflume"]) - 10.0)
    yr = dy2 + 1.0 + rng.random(n) * (width - 2.0)
    zr = 1.0 + rng.random(n)
    rel = pp["rr_s"] - pp["rr"][:, None, :]
    eps = rng.choice(np.array([-1e-6, -1e-9, -1e-12, -1e-15, 0.0, 1e-15, 1e-12, 1e-9, 1e-6]), n)
    kind = rng.integers(0, 3, n)   # 0 bed, 1 left wall, 2 right wall
    for i in range(n):
        q = np.array([xr[i], yr[i], zr[i]])
        # sphere offsets in the slope frame (a rotation of the lab offsets)
        o = np.stack([rel[i, :, 0] * cost - rel[i, :, 2] * sint, rel[i, :, 1],
                      rel[i, :, 0] * sint + rel[i, :, 2] * cost], 1)
        if kind[i] == 0:
            q[2] = rad * (1.0 + eps[i]) - o[:, 2].min()
        elif kind[i] == 1:
            q[1] = dy2 + rad * (1.0 + eps[i]) - o[:, 1].min()
        else:
            q[1] = dy2 + width - rad * (1.0 + eps[i]) - o[:, 1].max()
        pp["rr"][i] = [q[0] * cost + q[2] * sint, q[1], q[2] * cost - q[0] * sint]
    sphere_centres(pp)
    rotate_slope(pp, sys)
    _check(af3d, oracle, sys, fun, pp)
