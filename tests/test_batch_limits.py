"""Batch sizes the engine cannot address are refused at creation, before any
device memory is touched (so these run without a GPU): the sorted words
carry a bead's batch index in 29 bits, one system's grid has at most 1024
cells per side, and cells are addressed with 32-bit ints. Per-system arrays
of the wrong length are refused by the binding before the C call."""
import pytest

from tfm_gb300.ccpgpu import Batch, CcpError

PARAMS = "force_field baseline\n"


def test_too_many_beads():
    with pytest.raises(CcpError, match="more than 536870911 beads"):
        Batch(PARAMS, [1 << 28, 1 << 28])


def test_grid_side_limit():
    # 10 beads in a nucleus of radius 700: 1120 cells of 1.25 sigma per side
    with pytest.raises(CcpError, match="more than 1024 cells per side"):
        Batch(PARAMS, [10], radii=[700.0])


def test_total_cells_limit():
    # three grids of 800^3 cells each, twice over in the typed layout
    with pytest.raises(CcpError, match="cells; use a larger cell_side"):
        Batch(PARAMS, [10, 10, 10], radii=[500.0, 500.0, 500.0])



def test_per_system_arrays_must_match():
    for kw in (dict(n_chains=[1]), dict(radii=[5.0, 5.0, 5.0]), dict(seeds=[1])):
        with pytest.raises(ValueError, match="one entry per system"):
            Batch(PARAMS, [100, 200], **kw)
    with pytest.raises(ValueError, match="non-empty"):
        Batch(PARAMS, [])
