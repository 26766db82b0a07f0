"""Two-moment rain on the device against the oracle (GPU).

A developed storm (300 oracle steps of the benchmark configuration) goes on with two-moment rain, its drop number
started as the reference starts rain without one (Marshall-Palmer's, boundedNumber): one step and twenty steps of the
device against the oracle, every carried field and the drop number, the rain at the ground. The device's rain
processes are FP32 like the rest of its microphysics (their FP32 restatement is checked against the oracle's FP64 on
the CPU in tests/test_device_code_on_cpu.py); the bounds are the one-moment step's: 1e-5 relative L2 after a step
(the drop number 1e-4: its fall and the reflectivity limiter of each sub-step are FP32 too; the cold-pool indicator
3e-5), 1e-4 after twenty.
Then the reference's model test (rain2m.test.ts:66-78) on the device, two-moment rain with lightning together, and the
drop number through a state file.
"""
import dataclasses

import numpy as np
import pytest

import pyoracle as O
from parity import FLOOR, developed_state, rel_l2
from meteolab_gb300.grid import DEFAULT_GRID, create_grid
from meteolab_gb300.scenarios import CARRIED, CHARGES, RunSpec, baseline_run, marshall_palmer_number

pytestmark = pytest.mark.gpu
DT = 3.0
GRID = create_grid(DEFAULT_GRID)
FIELDS = tuple(CARRIED) + ("rainNumber",)


@pytest.fixture(scope="module")
def ctx():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import Context
    c = Context()
    yield c
    c.close()


@pytest.fixture(scope="module")
def storm2m():
    base = developed_state(baseline_run(GRID, seed=42), 300)
    f = dict(base.fields)
    f["rainNumber"] = marshall_palmer_number(f["rain"], np.repeat(np.asarray(base.env.rho), GRID.layer))
    sw = dataclasses.replace(base.switches, rain_moments=2)
    return RunSpec(GRID, base.env, sw, f, base.seed, "storm2m")


def compare(ctx, spec, steps):
    o = O.OracleModel(spec)
    r = ctx.create(spec)
    o.step(DT, steps)
    r.step(steps)
    got = r.read(list(FIELDS))
    errs = {k: rel_l2(got[k], o.get(k), FLOOR.get(k, 0.0)) for k in FIELDS}
    prec = rel_l2(r.columns()["precipitation"], o.get("precipitation"))
    r.retire()
    return errs, prec


def test_one_step_matches_the_oracle(ctx, storm2m):
    errs, prec = compare(ctx, storm2m, 1)
    print("\n2M one step: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()) + f", precipitation {prec:.2e}")
    for k, e in errs.items():
        # the cold-pool indicator takes the evaporation's cooling directly, and two-moment evaporation is a chain of
        # FP32 powers and roots of the drop size (measured 1.05e-5)
        assert e < (1e-4 if k == "rainNumber" else 3e-5 if k == "cold" else 1e-5), (k, e)
    assert prec < 1e-5


def test_twenty_steps_match_the_oracle(ctx, storm2m):
    errs, prec = compare(ctx, storm2m, 20)
    print("\n2M twenty steps: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()) + f", precipitation {prec:.2e}")
    for k, e in errs.items():
        assert e < 1e-4, (k, e)
    assert prec < 1e-4


def test_rain_shaft_in_the_model(ctx):
    """rain2m.test.ts:66-78: a 2 g/kg shaft from 2 to 4 km over a few columns; rain at the ground, the number in bounds;
    the rain at the ground and the fields against the oracle's (1e-4)."""
    base = baseline_run(GRID, seed=3, bubble=0.0)
    f = {k: v.copy() for k, v in base.fields.items()}
    f["rainNumber"] = np.zeros(GRID.n, np.float32)
    for z in range(GRID.nz):
        if 2000 < GRID.zs[z] < 4000:
            for c in range(6):
                i = c + z * GRID.layer
                f["rain"][i] = 2e-3
                f["rainNumber"][i] = O.r2m_bounded(2e-3, 0, base.env.rho[z])
    spec = RunSpec(GRID, base.env, dataclasses.replace(base.switches, rain_moments=2), f, 3, "shaft")
    r = ctx.create(spec)
    o = O.OracleModel(spec)
    r.step(200)
    o.step(DT, 200)
    prec = r.columns()["precipitation"]
    assert float(np.sum(prec)) > 0
    e = rel_l2(prec, o.get("precipitation"))
    errs = {k: rel_l2(r.read([k])[k], o.get(k), FLOOR.get(k, 0.0)) for k in ("rain", "rainNumber", "q", "theta")}
    print(f"\n2M shaft, 200 steps: precipitation {e:.2e}, " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    assert e < 1e-4 and all(v < 1e-4 for v in errs.values())
    got = r.read(["rain", "rainNumber"])
    xv_min, xv_max, _ = O.r2m_limits()
    assert (got["rainNumber"] >= 0).all()
    wet = got["rain"] > 1e-7
    xv = got["rain"][wet].astype(np.float64) / (1000 * got["rainNumber"][wet].astype(np.float64))
    assert (xv >= xv_min * .999).all() and (xv <= xv_max * 1.001).all()
    r.retire()


def test_with_lightning(ctx, storm2m):
    """Both extra sets together: an electrified two-moment run against the oracle over five steps (the charge on rain
    falls with the two-moment mass-weighted speed)."""
    spec = RunSpec(GRID, storm2m.env, dataclasses.replace(storm2m.switches, lightning=1), storm2m.fields, storm2m.seed, "storm2m+e")
    o = O.OracleModel(spec)
    r = ctx.create(spec)
    o.step(DT, 5)
    r.step(5)
    got = r.read(list(FIELDS) + list(CHARGES))
    errs = {k: rel_l2(got[k], o.get(k), FLOOR.get(k, 0.0)) for k in FIELDS}
    print("\n2M + lightning, five steps: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    for k, e in errs.items():
        assert e < 1e-4, (k, e)
    for k in CHARGES:
        a, b = got[k].astype(np.float64), o.get(k)
        assert np.linalg.norm(a - b) <= 1e-3 * max(np.linalg.norm(b), 1e-30) + 1e-12 * np.sqrt(a.size), k
    r.retire()


def test_drop_number_through_a_state_file(ctx, storm2m):
    import state_format as SF
    r = ctx.create(storm2m)
    r.step(2)
    img = r.save_state({"moments": 2}, persisted=0.0)
    _, fields, _ = SF.read_state(img)
    got = r.read(["rainNumber"])
    assert np.array_equal(fields["rainNumber"], got["rainNumber"])
    a = ctx.create(storm2m)
    a.load_state(img)
    assert np.array_equal(a.read(["rainNumber"])["rainNumber"], got["rainNumber"])
    assert a.save_state({"moments": 2}, persisted=0.0) == img
    r.retire()
    a.retire()
