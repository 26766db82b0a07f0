"""Saved state (.meteolab files) straight from and to device slots (GPU): the reference's state tests
(src/core/state.test.ts) through the C ABI, with the format's oracle (oracle/state_format.py) reading what the device
saves and writing what it loads.

The device keeps theta as its departure from the base profile; the file holds theta itself (FP32), so a run loaded
from a file continues the saved one to the rounding of theta (a few 1e-5 K), not bit for bit as the reference's
FP32-theta model does. Loading one file into two runs gives the same bits, and saving a loaded run gives the file back
byte for byte."""
import dataclasses

import numpy as np
import pytest

import state_format as SF
from parity import rel_l2
from meteolab_gb300.grid import DEFAULT_GRID, create_grid
from meteolab_gb300.scenarios import CARRIED, baseline_run

pytestmark = pytest.mark.gpu
CONFIG = {"seed": 7, "surfaceTemp": 30.0, "preset": "summer day", "nested": {"version": 9}}


@pytest.fixture(scope="module")
def ctx():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import Context
    c = Context()
    yield c
    c.close()


def small_grid():
    # state.test.ts:5: a 16 x 12 grid of the standard spacing
    return create_grid(dataclasses.replace(DEFAULT_GRID, nx=16, ny=12, width=16 * 1200.0, depth=12 * 1125.0))


@pytest.fixture(scope="module")
def saved(ctx):
    spec = baseline_run(small_grid(), seed=7)
    r = ctx.create(spec)
    r.step(200)                       # 600 s, as state.test.ts:10
    img = r.save_state(CONFIG, persisted=12.0)
    return spec, r, img


def test_the_saved_image_is_the_run(ctx, saved):
    spec, r, img = saved
    header, fields, cols = SF.read_state(img)
    assert header["format"] == "meteolab-state" and header["version"] == 5
    assert header["config"] == CONFIG and header["time"] == 600 and header["persisted"] == 12
    assert (header["nx"], header["ny"], header["nz"]) == (16, 12, spec.grid.nz)
    state = r.read()
    for k in CARRIED:
        assert np.array_equal(fields[k], state[k]), k
    for k in ("chargeIce", "chargeGraupel", "chargeRain", "chargeAir", "rainNumber", "graupelNumber", "graupelVolume",
              "hailNumber", "hailVolume"):
        assert not fields[k].any(), k
    got = r.columns()
    for k in SF.STATE_COLUMNS:
        assert np.array_equal(cols[k], got[k]), k
    assert state["cloud"].max() > 0 and header["water"]["condensed"] > 0  # a growing storm, not an empty state


def test_a_loaded_run_continues_the_saved_one(ctx, saved):
    spec, r, img = saved
    a, b = ctx.create(spec), ctx.create(spec)
    info = a.load_state(img)
    b.load_state(img)
    assert info["time"] == 600 and a.time == 600
    # the file gives back the run's fields as read (theta too: the departure the device keeps rounds back to it)
    x, y = a.read(), r.read()
    for k in CARRIED:
        assert np.array_equal(x[k], y[k]), k
    # saving the loaded run gives the file back byte for byte
    assert a.save_state(CONFIG, persisted=12.0) == img
    # five more steps (state.test.ts:17): the two loaded runs bit for bit, the original to the rounding of theta
    for m in (r, a, b):
        m.step(5)
    x, y, z = a.read(), b.read(), r.read()
    worst = 0.0
    for k in CARRIED:
        assert np.array_equal(x[k], y[k]), k
        worst = max(worst, rel_l2(x[k], z[k], 1e-9))
    print(f"\nloaded vs saved run after 5 steps: worst rel-L2 {worst:.2e}")
    assert worst < 1e-4
    assert np.array_equal(a.columns()["precipitation"], b.columns()["precipitation"])
    a.retire(); b.retire()


def test_an_old_file_loads_with_the_missing_fields_zero(ctx):
    # state.test.ts:41-50: a version 1 file, every value 1: the hail is 1, what version 1 lacks is zero
    spec = baseline_run(small_grid(), seed=3)
    g = spec.grid
    img = SF.save_state({k: np.ones(g.n, np.float32) for k in SF.STATE_FIELDS}, {k: np.ones(g.layer, np.float32) for k in SF.STATE_COLUMNS},
                        {}, 60, 0, g.nx, g.ny, g.nz, version=1)
    r = ctx.create(spec)
    r.write({"iceNumber": np.full(g.n, 5.0, np.float32)})
    info = r.load_state(img)
    assert info["version"] == 1 and r.time == 60
    f = r.read()
    assert (f["hail"] == 1).all() and (f["rain"] == 1).all() and not f["iceNumber"].any()
    assert np.max(np.abs(f["theta"] - 1)) < 1e-4
    assert (r.columns()["hailSize"] == 1).all()
    r.retire()


def test_refuses_a_file_of_another_grid_and_a_damaged_one(ctx, saved):
    from meteolab_gb300.runtime import StormGpuError
    spec, r, img = saved
    other = ctx.create(baseline_run(create_grid(DEFAULT_GRID), seed=1))
    with pytest.raises(StormGpuError, match=r"the file's grid is 16x12x\d+, the run's 40x32x\d+"):
        other.load_state(img)
    with pytest.raises(StormGpuError, match="the file's size does not match the grid"):
        r.load_state(img[:-4])
    with pytest.raises(StormGpuError, match="this is not a MeteoLab state file"):
        r.load_state(b"hello world, not a state")
    other.retire()


def test_the_saved_water_start_is_the_initial_reservoirs(ctx, saved):
    """water.start in the saved header is waterReservoirs of the run's initial fields (src/core/model.ts:450,
    src/core/water.ts:27-46: vapour above the profile, condensate and precipitation aloft, each by the level's air
    mass), FP64; a run loaded from the file saves the same start again."""
    spec, r, img = saved
    header, _, _ = SF.read_state(img)
    g, env, f = spec.grid, spec.env, spec.fields
    want = 0.0
    for z in range(g.nz):
        sl = slice(z * g.layer, (z + 1) * g.layer)
        mass = env.rho[z] * g.dx * g.dy * g.hz[z]
        v = np.sum(f["q"][sl].astype(np.float64) - env.q[z])
        c = np.sum(f["cloud"][sl].astype(np.float64) + f["ice"][sl])
        a = np.sum(f["rain"][sl].astype(np.float64) + f["snow"][sl] + f["graupel"][sl] + f["hail"][sl])
        want += (v + c + a) * mass
    start = header["water"]["start"]
    assert abs(start - want) <= 1e-9 * max(1.0, abs(want)), (start, want)
    other = ctx.create(spec)
    other.load_state(img)
    again, _, _ = SF.read_state(other.save_state(CONFIG, persisted=12.0))
    assert again["water"]["start"] == start
    other.retire()
