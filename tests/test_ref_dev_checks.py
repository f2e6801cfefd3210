"""Host-side bounds checks of the reference device-kernel driver (oracle/ref_dev.py), on the CPU:
the reference's cell_locate_dev (cells.cu:150-202) writes outside cell_vec for a clump off the
grid or a cell holding more than ntags clumps, so the driver measures both before every launch
and refuses a state that is not safely inside."""
import numpy as np
import pytest

from oracle import ref_dev
from oracle.pyoracle import CELL_PAR, PARTICLE, SYSTEM_PAR


def _grid(ncell=(10, 6, 4), side=0.5, lo=(0.0, 1.0, 2.0), ntags=8):
    cp = np.zeros((), dtype=CELL_PAR)
    cp["ntags"] = ntags
    cp["ncell"] = ncell
    cp["ncell3"] = int(np.prod(ncell))
    cp["ntot"] = int(np.prod(ncell)) * ntags
    cp["cell_side"] = side
    cp["cs_inv"] = 1.0 / side
    cp["rr_min"] = lo
    cp["rr_max"] = np.asarray(lo) + side * np.asarray(ncell)
    return cp


def _state(points, time=0.0, side_x=100.0):
    pp = np.zeros(len(points), dtype=PARTICLE)
    pp["rr"] = points
    sys = np.zeros((), dtype=SYSTEM_PAR)
    sys["npart"] = len(points)
    sys["time"] = time
    sys["side"] = (side_x, 0.0, 0.0)
    return pp, sys


def test_grid_margin_in_cells():
    cp = _grid()
    # x = 0.75 is 1.5 cells from the low face; y = 1.25 is 0.5 cells; z = 3.9 is 0.2 cells from the top
    pp, sys = _state([[0.75, 2.0, 3.0], [2.0, 1.25, 3.0], [2.0, 2.0, 3.9]])
    assert ref_dev.grid_margin(pp[:1], cp, sys) == pytest.approx(1.5)
    assert ref_dev.grid_margin(pp[:2], cp, sys) == pytest.approx(0.5)
    assert ref_dev.grid_margin(pp, cp, sys) == pytest.approx(0.2)
    out, _ = _state([[-0.1, 2.0, 3.0]])
    assert ref_dev.grid_margin(out, cp, sys) < 0


def test_removed_clumps_are_not_binned():
    cp = _grid()
    # far outside the grid but past side.x after the door opened (time > 0): skipped (cells.cu:171)
    pp, sys = _state([[50.0, 2.0, 3.0], [1.0, 2.0, 3.0]], time=1e-3, side_x=20.0)
    assert ref_dev.grid_margin(pp, cp, sys) == pytest.approx(2.0)
    assert ref_dev.max_occupancy(pp, cp, sys) == 1
    pp0, sys0 = _state([[50.0, 2.0, 3.0], [1.0, 2.0, 3.0]], time=0.0, side_x=20.0)
    assert ref_dev.grid_margin(pp0, cp, sys0) < 0   # at time 0 every clump is binned


def test_max_occupancy_uses_cell_locate_arithmetic():
    cp = _grid()
    # three clumps in cell (1, 2, 1), one in (2, 2, 1); x = 5.0 is exactly ncell.x: cell 9
    pts = [[0.6, 2.1, 2.6], [0.9, 2.4, 2.9], [0.51, 2.01, 2.51], [1.1, 2.2, 2.7], [5.0, 2.0, 3.0]]
    pp, sys = _state(pts)
    assert ref_dev.max_occupancy(pp, cp, sys) == 3


@pytest.mark.skipif(not ref_dev.available(), reason="reference device kernels not built")
def test_driver_refuses_unsafe_states():
    cp = _grid(ntags=4)
    sys = np.zeros((), dtype=SYSTEM_PAR)
    fun = np.zeros((), dtype=ref_dev.FUNNEL)
    off, s = _state([[-0.2, 2.0, 3.0]])
    with pytest.raises(ValueError, match="not safely inside the grid"):
        ref_dev.RefDeviceRun(s, fun, cp, off)
    full, s = _state([[0.6, 2.1, 2.6], [0.9, 2.4, 2.9], [0.51, 2.01, 2.51]])
    with pytest.raises(ValueError, match="fullest cell 3 of 4"):
        ref_dev.RefDeviceRun(s, fun, cp, full)
