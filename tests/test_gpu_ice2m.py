"""Two-moment graupel and hail on the device against the oracle (GPU).

A mature storm (600 oracle steps, 30 minutes, of the benchmark configuration: some 10 g/kg of graupel, 7 g/kg of hail
and hail at the ground) goes on with the reference's two-moment
configuration (SimConfig.moments 2: two-moment rain and two-moment graupel and hail, src/core/model.ts:331): the drop
number started as the reference starts rain without one (Marshall-Palmer's), graupel's and hail's number and volume as
the one-moment classes of the same mass. One step and twenty steps of the device against the oracle, every carried
field, the numbers and volumes, the rain at the ground and the hail swath. The device's graupel and hail processes are
FP32 like the rest of its microphysics (checked against the oracle's FP64 on the CPU in
tests/test_device_code_on_cpu.py); the bounds are those of two-moment rain: 1e-5 relative L2 for the base fields after
a step (the numbers and volumes 1e-4: their fall and limiter of each sub-step are FP32 too), 1e-4 after twenty.
Then the reference's model test (ice2m.test.ts:66-80) on the device, two-moment ice with lightning (the charging by the
classes' own moments), and the numbers and volumes through a state file.
"""
import dataclasses

import numpy as np
import pytest

import pyoracle as O
from parity import FLOOR, developed_state, rel_l2
from meteolab_gb300.grid import DEFAULT_GRID, create_grid
from meteolab_gb300.scenarios import CARRIED, CHARGES, ICE2M, RunSpec, baseline_run, exponential_ice_moments, marshall_palmer_number

pytestmark = pytest.mark.gpu
DT = 3.0
GRID = create_grid(DEFAULT_GRID)
FIELDS = tuple(CARRIED) + ("rainNumber",) + tuple(ICE2M)
SCALE_FLOOR = {"graupelNumber": 1e-3, "hailNumber": 1e-3, "graupelVolume": 1e-12, "hailVolume": 1e-12}


@pytest.fixture(scope="module")
def ctx():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import Context
    c = Context()
    yield c
    c.close()


def two_moment(base: RunSpec, label: str) -> RunSpec:
    f = dict(base.fields)
    rho = np.repeat(np.asarray(base.env.rho), GRID.layer)
    f["rainNumber"] = marshall_palmer_number(f["rain"], rho)
    for kind in ("graupel", "hail"):
        f[kind + "Number"], f[kind + "Volume"] = exponential_ice_moments(f[kind], rho, kind)
    sw = dataclasses.replace(base.switches, rain_moments=2, ice_moments=2)
    return RunSpec(GRID, base.env, sw, f, base.seed, label)


@pytest.fixture(scope="module")
def storm():
    return two_moment(developed_state(baseline_run(GRID, seed=42), 600), "storm2m-ice")


def err(got, ref, k):
    return rel_l2(got, ref, FLOOR.get(k, SCALE_FLOOR.get(k, 0.0)))


def compare(ctx, spec, steps, fields=FIELDS):
    o = O.OracleModel(spec)
    r = ctx.create(spec)
    o.step(DT, steps)
    r.step(steps)
    got = r.read(list(fields))
    errs = {k: err(got[k], o.get(k), k) for k in fields}
    cols = r.columns()
    col_errs = {k: rel_l2(cols[k], o.get(k)) for k in ("precipitation", "hailGround", "hailSize")}
    r.retire()
    return errs, col_errs


def report(title, errs, cols):
    print(f"\n{title}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()) + "; " + ", ".join(f"{k} {v:.2e}" for k, v in cols.items()))


def test_one_step_matches_the_oracle(ctx, storm):
    errs, cols = compare(ctx, storm, 1)
    report("2M ice, one step", errs, cols)
    for k, e in errs.items():
        assert e < (1e-4 if k in ICE2M or k == "rainNumber" else 3e-5 if k == "cold" else 1e-5), (k, e)
    assert all(v < 1e-5 for v in cols.values()), cols


def ulp_spread(spec, steps):
    """The oracle's own distance after `steps` steps from its run with theta moved by one FP32 ulp (up or down at random)
    at every node: how far the reference algorithm carries a rounding-sized difference in this state."""
    f = dict(spec.fields)
    th = np.asarray(f["theta"], np.float32)
    up = np.random.default_rng(0).random(th.size) < .5
    f["theta"] = np.nextafter(th, np.where(up, np.inf, -np.inf).astype(np.float32)).astype(np.float32)
    a, b = O.OracleModel(spec), O.OracleModel(RunSpec(spec.grid, spec.env, spec.switches, f, spec.seed, spec.label + "+ulp"))
    a.step(DT, steps)
    b.step(DT, steps)
    return {k: err(b.get(k), a.get(k), k) for k in FIELDS}


def test_twenty_steps_match_the_oracle(ctx, storm):
    """Over twenty steps the two-moment graupel's wet or dry growth (a switch: its particles soak to 900 kg/m3 or take the
    rime's density, which sets how well they collect snow a step later) carries rounding-sized differences into snow and
    the drop number: the oracle's own run from a theta one ulp away ends 1e-3 from it in snow, 4e-4 in the drop number
    (the one-moment and two-moment-rain steps under 1e-5). Each field's bound is 1e-4 or four times that spread."""
    errs, cols = compare(ctx, storm, 20)
    spread = ulp_spread(storm, 20)
    report("2M ice, twenty steps", errs, cols)
    print("  the oracle's one-ulp spread: " + ", ".join(f"{k} {v:.2e}" for k, v in spread.items()))
    for k, e in errs.items():
        assert e < max(1e-4, 4 * spread[k]), (k, e, spread[k])
    assert all(v < 1e-4 for v in cols.values()), cols


def test_graupel_and_hail_shafts_in_the_model(ctx):
    """ice2m.test.ts:66-80: graupel (2 g/kg, 2000 per kg at 500 kg/m3) and hail (1 g/kg, 50 per kg at 900 kg/m3) from 3
    to 7 km over eight columns for 120 steps: precipitation at the ground, numbers finite and non-negative, where there
    is mass a number and a density of 160-910 kg/m3; the fields and the ground columns against the oracle's (1e-4)."""
    base = baseline_run(GRID, seed=5)
    f = {k: v.copy() for k, v in base.fields.items()}
    for k in ("rainNumber",) + ICE2M:
        f[k] = np.zeros(GRID.n, np.float32)
    for z in range(GRID.nz):
        if 3000 < GRID.zs[z] < 7000:
            for c in range(8):
                i = c + z * GRID.layer
                f["graupel"][i], f["graupelNumber"][i], f["graupelVolume"][i] = 2e-3, 2e3, 2e-3 / 500
                f["hail"][i], f["hailNumber"][i], f["hailVolume"][i] = 1e-3, 50, 1e-3 / 900
    spec = RunSpec(GRID, base.env, dataclasses.replace(base.switches, rain_moments=2, ice_moments=2), f, 5, "ice2m-shafts")
    r = ctx.create(spec)
    o = O.OracleModel(spec)
    r.step(120)
    o.step(DT, 120)
    cols = r.columns()
    assert float(np.sum(cols["precipitation"])) > 0
    got = r.read(list(FIELDS))
    errs = {k: err(got[k], o.get(k), k) for k in ("graupel", "hail", "rain", "q", "theta") + ICE2M}
    cerrs = {k: rel_l2(cols[k], o.get(k)) for k in ("precipitation", "hailGround", "hailSize")}
    report("2M ice shafts, 120 steps", errs, cerrs)
    assert all(v < 1e-4 for v in errs.values()) and all(v < 1e-4 for v in cerrs.values())
    for q, n, v in (("graupel", "graupelNumber", "graupelVolume"), ("hail", "hailNumber", "hailVolume")):
        assert np.isfinite(got[n]).all() and (got[n] >= 0).all()
        big = got[q] > 1e-7
        assert (got[n][big] > 0).all()
        d = got[q][big] / got[v][big]
        assert (d > 160).all() and (d < 910).all()
    r.retire()


def test_with_lightning(ctx, storm):
    """Two-moment graupel and hail charge by their own moments (model.ts:1461-1466): an electrified two-moment run
    against the oracle over five steps, each field within 1e-4 or four times the oracle's own one-ulp spread (snow: see
    test_twenty_steps_match_the_oracle), the charge carriers to 1e-3 as the one-moment electrified step."""
    spec = RunSpec(GRID, storm.env, dataclasses.replace(storm.switches, lightning=1), storm.fields, storm.seed, "storm2m-ice+e")
    o = O.OracleModel(spec)
    r = ctx.create(spec)
    o.step(DT, 5)
    r.step(5)
    got = r.read(list(FIELDS) + list(CHARGES))
    errs = {k: err(got[k], o.get(k), k) for k in FIELDS}
    spread = ulp_spread(spec, 5)
    print("\n2M ice + lightning, five steps: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    print("  the oracle's one-ulp spread: " + ", ".join(f"{k} {v:.2e}" for k, v in spread.items()))
    for k, e in errs.items():
        assert e < max(1e-4, 4 * spread[k]), (k, e, spread[k])
    for k in CHARGES:
        a, b = got[k].astype(np.float64), o.get(k)
        assert np.linalg.norm(a - b) <= 1e-3 * max(np.linalg.norm(b), 1e-30) + 1e-12 * np.sqrt(a.size), k
    r.retire()


def test_numbers_and_volumes_through_a_state_file(ctx, storm):
    import state_format as SF
    r = ctx.create(storm)
    r.step(2)
    img = r.save_state({"moments": 2}, persisted=0.0)
    _, fields, _ = SF.read_state(img)
    got = r.read(list(ICE2M))
    for k in ICE2M:
        assert np.array_equal(fields[k], got[k]), k
    a = ctx.create(storm)
    a.load_state(img)
    back = a.read(list(ICE2M))
    assert all(np.array_equal(back[k], got[k]) for k in ICE2M)
    assert a.save_state({"moments": 2}, persisted=0.0) == img
    r.retire()
    a.retire()


def test_mixed_batch_gives_each_run_its_own_bits(ctx, storm):
    """A one-moment run, a two-moment run (rain, graupel and hail) and an electrified two-moment run stepped together in
    one batch (one plan: the extras' kernels, the two-moment fall and the lightning beside the plain run's work) give
    each run exactly the fields, numbers and charges it has stepped alone."""
    plain = RunSpec(GRID, storm.env, dataclasses.replace(storm.switches, rain_moments=1, ice_moments=1),
                    {k: v for k, v in storm.fields.items() if k in CARRIED}, storm.seed, "plain")
    elec = RunSpec(GRID, storm.env, dataclasses.replace(storm.switches, lightning=1), storm.fields, storm.seed, "storm2m-ice+e")
    specs = (plain, storm, elec)
    names = (list(CARRIED), list(FIELDS), list(FIELDS) + list(CHARGES))
    alone = []
    for s, nm in zip(specs, names):
        r = ctx.create(s)
        r.step(3)
        alone.append(r.read(nm))
        r.retire()
    runs = [ctx.create(s) for s in specs]
    ctx.batch_step(runs, 3)
    for r, a, nm in zip(runs, alone, names):
        b = r.read(nm)
        assert r.status()["failed"] == 0
        for k in nm:
            assert np.array_equal(a[k], b[k]), (r.spec.label, k)
        r.retire()
