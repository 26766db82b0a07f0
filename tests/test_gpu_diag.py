"""Per-run diagnostics on the device (GPU): the rotation tracking after every step (updateRotation), the swaths
(addSwaths) and a sample's diagnostics(), through the C ABI: the reference's own cases (src/core/model.test.ts:25-55),
parity with the oracle's restatement on the same fields (a developed storm), the swaths against their definition
step by step, and independence of the batch.

Tolerances: the device sums w zeta hz over the 2-5 km levels in FP32 (the reference in FP64): the UH values and the
core vorticity to 1e-4 relative; maxima of fields, counts and columns exactly."""
import dataclasses

import numpy as np
import pytest

import pyoracle as O
from parity import developed_state, threads
from test_oracle_diag import cores_fields, vortex_fields
from meteolab_gb300.grid import DEFAULT_GRID, LARGE_GRID, create_grid
from meteolab_gb300.scenarios import CARRIED, baseline_run

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import Context
    c = Context()
    yield c
    c.close()


@pytest.fixture(scope="module")
def storm():
    return developed_state(baseline_run(create_grid(DEFAULT_GRID), seed=42), 300)


def close(a, b, rel=1e-4, abs_=1e-6):
    return abs(a - b) <= rel * max(abs(a), abs(b)) + abs_


def test_counts_updraught_cores_by_height(ctx):
    spec = baseline_run(create_grid(DEFAULT_GRID), seed=1)
    r = ctx.create(spec)
    r.write({k: a.astype(np.float32) for k, a in cores_fields(spec.grid).items()})
    assert r.diagnostics()["cores"] == 2
    r.retire()


def test_tells_a_rotating_updraught_from_a_vortex_pair(ctx):
    spec = baseline_run(create_grid(DEFAULT_GRID), seed=1)
    r = ctx.create(spec)
    r.write({k: a.astype(np.float32) for k, a in vortex_fields(spec.grid, [(0, .02)]).items()})
    r.refresh_rotation()
    meso = r.rotation()
    r.write({k: a.astype(np.float32) for k, a in vortex_fields(spec.grid, [(-3, .02), (3, -.02)]).items()})
    r.refresh_rotation()
    pair = r.rotation()
    assert meso["coreZeta"] > .004
    assert pair["uh"] > 200 and pair["anticyclonic"] > 200
    assert abs(pair["coreZeta"]) < .002
    r.retire()


def oracle_on(run, spec):
    """The oracle holding the device run's fields (FP64 model) and its rain gauge."""
    m = O.OracleModel(spec, fp64=True, threads=threads())
    for k, a in run.read().items():
        m.set(k, a.astype(np.float64))
    m.set("precipitation", run.columns()["precipitation"].astype(np.float64))
    return m


def test_rotation_and_diagnostics_match_the_oracle_on_a_storm(ctx, storm):
    r = ctx.create(storm)
    r.step(400)  # 35 minutes in: rain on the ground, updraught cores
    got, col = r.rotation(column=True)
    m = oracle_on(r, storm)
    m.update_rotation(0)
    ref, rcol = m.rotation()
    print("\ndevice rotation:", {k: round(v, 5) for k, v in got.items()})
    print("oracle rotation:", {k: round(v, 5) for k, v in ref.items()})
    assert np.max(np.abs(col - rcol)) <= 1e-4 * max(1.0, np.max(np.abs(rcol)))
    for k in ("uh", "anticyclonic", "uh01", "uh03", "coreZeta", "coreUH", "coreAnti"):
        assert close(got[k], ref[k]), (k, got[k], ref[k])
    for k in ("x", "y", "low"):
        assert got[k] == ref[k], (k, got[k], ref[k])
    assert got["uh"] > 0 and got["time"] == pytest.approx(400 * storm.switches.dt)
    d, rd = r.diagnostics(), m.diagnostics()
    print("device diagnostics:", {k: round(v, 5) for k, v in d.items()})
    print("oracle diagnostics:", {k: round(v, 5) for k, v in rd.items()})
    for k in ("updraft", "downdraft", "maxCloud", "coldMax", "gust", "rainTotal", "cores", "cloudTop", "thermalTop"):
        assert close(d[k], rd[k], 1e-6), (k, d[k], rd[k])
    for k in ("rainRate", "hail", "outflow", "outflowLow"):
        assert close(d[k], rd[k], 1e-4, 1e-5), (k, d[k], rd[k])
    assert d["updraft"] > 10 and d["cores"] >= 1 and d["rainRate"] > 0 and got["coreZeta"] != 0
    r.retire()


def test_swaths_are_the_maxima_of_every_step(ctx, storm):
    # a moving domain (5 m/s east, 2 m/s south): each step folds onto the ground shifted by the motion so far
    spec = dataclasses.replace(storm, switches=dataclasses.replace(storm.switches, frame_u=5.0, frame_v=-2.0))
    r = ctx.create(spec)
    g = spec.grid
    gust, uhm = np.zeros(g.layer, np.float32), np.zeros(g.layer, np.float32)
    dt = spec.switches.dt
    for s in range(1, 13):
        r.step(1)
        rot, col = r.rotation(column=True)
        f = r.read(["u", "v"])
        t = s * dt
        sx, sy = int(np.floor(5.0 * t / g.dx + .5)), int(np.floor(-2.0 * t / g.dy + .5))
        x, y = np.meshgrid(np.arange(g.nx), np.arange(g.ny))
        dest = ((x + sx) % g.nx + g.nx * ((y + sy) % g.ny)).ravel()
        wind = np.sqrt((f["u"][:g.layer] + np.float32(5.0)) ** 2 + (f["v"][:g.layer] + np.float32(-2.0)) ** 2).astype(np.float32)
        np.maximum.at(gust, dest, wind)
        np.maximum.at(uhm, dest, col)
    sw = r.swaths()
    assert np.allclose(sw["gustMax"], gust, rtol=1e-6, atol=1e-6)
    assert np.array_equal(sw["uhMax"], uhm)
    r.reset_swaths()
    assert not r.swaths()["gustMax"].any()
    r.retire()


def test_rotation_is_the_same_alone_and_in_a_batch(ctx, storm):
    alone = ctx.create(storm)
    alone.step(6)
    a, acol = alone.rotation(column=True)
    x, y = ctx.create(storm), ctx.create(baseline_run(create_grid(LARGE_GRID), seed=9))
    ctx.batch_step([x, y], 6)
    b, bcol = x.rotation(column=True)
    assert a == b and np.array_equal(acol, bcol)
    assert np.array_equal(alone.swaths()["uhMax"], x.swaths()["uhMax"])
    for run in (alone, x, y):
        run.retire()


def test_a_loaded_state_keeps_the_rotation_time(ctx, storm):
    r = ctx.create(storm)
    r.step(10)
    img = r.save_state({"seed": 42})
    before = r.rotation()
    s = ctx.create(storm)
    s.load_state(img)
    after = s.rotation()
    assert after["persisted"] == before["persisted"] and after["time"] == before["time"]
    assert after["uh"] == before["uh"] and after["coreZeta"] == before["coreZeta"]
    r.retire(); s.retire()


def test_members_sample_every_minute_and_a_batch_gives_each_members_own_result(ctx):
    # ensemble.test.ts:16-21: a member runs for 3 minutes: samples at 0, 1, 2, 3 minutes and a surface wind swath
    from meteolab_gb300.ensemble import SAMPLE_EVERY, run_members
    from meteolab_gb300.scenarios import ensemble_members
    specs = ensemble_members(create_grid(DEFAULT_GRID), 3, seed=11)
    res = run_members(ctx, specs, 3)
    for r in res:
        assert [s["t"] for s in r["samples"]] == [k * SAMPLE_EVERY for k in range(4)]
        assert r["gustMax"].shape == (r["nx"] * r["ny"],) and r["gustMax"].max() > 0
    alone = run_members(ctx, specs[1:2], 3)[0]
    assert alone["samples"] == res[1]["samples"]
    for k in ("rainTotal", "hailSize", "gustMax", "uhMax"):
        assert np.array_equal(alone[k], res[1][k]), k
