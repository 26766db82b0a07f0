"""The library's terrain geometry (sg_terrain_heights, sg_terrain_geometry: host arithmetic, no device) against the
oracle's restatement of src/core/terrain.ts, bit for bit, and the reference's own assertions on it
(src/core/terrain.test.ts:10-21, :178-198) through the C ABI. The masked projection that builds on this geometry is
checked on the device in test_gpu_terrain.py."""
import numpy as np
import pytest

import pyoracle as O
from meteolab_gb300 import runtime as R
from meteolab_gb300.grid import DEFAULT_GRID, GridOptions, create_grid

TEST_GRID = create_grid(GridOptions(32, 24, 30, 38_400, 28_800, 15_000, bottom_spacing=100))
FORMS = (("hill", 1, 5, {}), ("ridge", .8, 4, {"heading": 30}), ("plateau", .5, 8, {"x": 10, "y": 7}),
         ("schar", .4, 5, {"wavelength": 3}), ("hill", 2.5, 1, {"x": 3, "y": 30}))


@pytest.fixture(scope="module", autouse=True)
def library():
    from meteolab_gb300 import build
    build.build()


@pytest.mark.parametrize("grid", [TEST_GRID, create_grid(DEFAULT_GRID)], ids=["32x24x30", "40x32x50"])
@pytest.mark.parametrize("form", FORMS, ids=[f[0] + str(i) for i, f in enumerate(FORMS)])
def test_geometry_matches_the_oracle_bit_for_bit(grid, form):
    kind, height, width, extra = form
    mine = R.terrain_heights(dict(kind=kind, height=height, width=width, **extra), grid)
    theirs = O.terrain_heights(grid, kind, height, width, **extra)
    assert np.array_equal(mine, theirs)
    a, b = R.terrain_geometry(grid, mine), O.terrain_geometry(grid, theirs)
    for key in ("solid", "levels", "heights", "ax", "ay", "slope"):
        assert np.array_equal(a[key], b[key]), key


def test_the_reference_heights_through_the_abi():  # terrain.test.ts:10-21
    nx, ny = TEST_GRID.nx, TEST_GRID.ny
    hill = R.terrain_heights({"kind": "hill", "height": 1, "width": 5}, TEST_GRID)
    top = float(hill.max())
    assert 800 < top <= 1000 and hill[0] < .15 * top
    ridge = R.terrain_heights({"kind": "ridge", "height": .8, "width": 4}, TEST_GRID)
    assert all(abs(float(ridge[nx // 2 + nx * j]) - float(ridge[nx // 2])) < 5e-4 for j in range(1, ny))
    plateau = R.terrain_heights({"kind": "plateau", "height": .5, "width": 8}, TEST_GRID)
    assert plateau[nx // 2 + nx * (ny // 2)] > 450 and plateau[0] < 50


def test_the_reference_apertures_through_the_abi():  # terrain.test.ts:178-198
    nx, nz, layer = TEST_GRID.nx, TEST_GRID.nz, TEST_GRID.nx * TEST_GRID.ny
    level = np.arange(layer * nz) // layer
    hz = np.asarray(TEST_GRID.hz)
    plain = R.terrain_geometry(TEST_GRID, np.zeros(layer, np.float32))
    assert (plain["ax"] == hz[level]).all() and (plain["ay"] == hz[level]).all()
    ramp = (37 * (np.arange(layer) % nx)).astype(np.float32)
    geo = R.terrain_geometry(TEST_GRID, ramp)
    ax, ay, lid = geo["ax"].reshape(nz, layer), geo["ay"].reshape(nz, layer), TEST_GRID.zs[nz - 1]
    c = np.arange(layer - 1)
    c = c[c % nx != nx - 1]
    assert np.abs(ax.sum(0)[c] - (lid - (ramp[c].astype(float) + ramp[c + 1]) / 2)).max() < 5e-7
    assert np.abs(ay.sum(0)[c] - (lid - ramp[c].astype(float))).max() < 5e-7


def test_bad_arguments_are_refused():
    g, keep = R._grid_struct(TEST_GRID)
    out = np.zeros(TEST_GRID.nx * TEST_GRID.ny, np.float32)
    bad = R.SgTerrain(7, 0, 1.0, 5.0, *[float("nan")] * 4)
    import ctypes as C
    assert R.load().sg_terrain_heights(C.byref(g), C.byref(bad), out.ctypes.data_as(C.POINTER(C.c_float))) == 1
    assert R.load().sg_terrain_geometry(C.byref(g), None, None, None, None, None, None, None) == 1
