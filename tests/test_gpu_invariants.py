"""The reference's invariant tests (src/core/invariants.test.ts) on the device step at full size (the standard
40x32x50 grid), and the device step against the committed golden vectors (tests/golden/step_small.npz).

Thresholds are the reference's; the oracle passes the same checks in tests/test_oracle_invariants.py.
"""
import os

import numpy as np
import pytest

from parity import FLOOR, WATER, dual_divergence, level_mean, rel_l2, water_total
from meteolab_gb300.environment import Environment, SliderConfig
from meteolab_gb300.grid import DEFAULT_GRID, create_grid
from meteolab_gb300.scenarios import CARRIED, RunSpec, Switches, baseline_profile, baseline_run, initial_fields

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "step_small.npz")


@pytest.fixture(scope="module")
def ctx():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import Context
    c = Context(0)
    yield c
    c.close()


def quiet_run(grid):
    env = Environment(SliderConfig(), grid, baseline_profile())
    return RunSpec(grid, env, Switches(), initial_fields(grid, env, 1, bubble=0.0, noise=0.0), 1, "quiet")


def test_background_state_holds_for_3_hours(ctx):  # invariants.test.ts:15-35
    spec = quiet_run(create_grid(DEFAULT_GRID))
    r = ctx.create(spec)
    r.step(3600)
    f = r.read(("theta", "u", "v", "q"))
    g, env = spec.grid, spec.env
    nz = g.nz
    assert max(abs(level_mean(f["theta"], g, z) - env.theta[z]) for z in range(nz)) < 0.05
    assert max(abs(level_mean(f["u"], g, z) - env.u[z]) for z in range(nz)) < 0.05
    assert max(abs(level_mean(f["v"], g, z) - env.v[z]) for z in range(nz)) < 0.05
    assert max(abs(level_mean(f["q"], g, z) - env.q[z]) for z in range(nz)) / env.q[0] < 0.01
    assert not r.status()["failed"]
    r.retire()


def test_final_projection_removes_uniform_vertical_velocity(ctx):  # invariants.test.ts:40-47
    spec = quiet_run(create_grid(DEFAULT_GRID))
    g = spec.grid
    fields = dict(spec.fields)
    fields["u"] = np.zeros(g.n, np.float32); fields["v"] = np.zeros(g.n, np.float32)
    w = np.zeros(g.n, np.float32); w[g.layer:(g.nz - 1) * g.layer] = 0.01
    fields["w"] = w
    spec = RunSpec(g, spec.env, spec.switches, fields, 1, "uniform w")
    r = ctx.create(spec)
    r.debug_part(5)
    w = r.read(("w",))["w"]
    for z in range(1, g.nz - 1):
        assert abs(level_mean(w, g, z)) < 1e-4
    r.retire()


@pytest.fixture(scope="module")
def storm(ctx):
    spec = baseline_run(create_grid(DEFAULT_GRID), seed=3, bubble=3.0, qv_max=0.016)
    r = ctx.create(spec)
    f0 = r.read(WATER)
    before = water_total(f0, np.zeros(spec.grid.layer), spec)
    r.step(300)  # 15 minutes
    yield spec, r, before
    r.retire()


def test_no_dual_cell_divergence_after_a_stormy_step(storm):  # invariants.test.ts:49-59
    spec, r, _ = storm
    f = r.read(("u", "v", "w"))
    div = dual_divergence(f["u"], f["v"], f["w"], spec.grid, spec.env.rho)
    assert np.max(np.abs(div)) < 1e-7
    assert r.status()["clipped"] == 0


def test_water_is_conserved_within_001_percent_in_a_30_minute_storm(storm):  # invariants.test.ts:84-94
    spec, r, before = storm
    r.step(300)  # to 30 minutes
    f = r.read(WATER)
    assert float(np.max(f["ice"])) > 1e-6 and float(np.max(f["graupel"])) > 1e-4
    after = water_total(f, r.columns()["precipitation"], spec)
    assert abs(after / before - 1) < 1e-4


def test_device_step_matches_golden_vectors(ctx):
    """From the golden developed state of the small grid, two device steps match the golden FP64 result."""
    import importlib.util
    spec_mod = importlib.util.spec_from_file_location("make_golden", os.path.join(os.path.dirname(GOLDEN), "make_golden.py"))
    mg = importlib.util.module_from_spec(spec_mod)
    spec_mod.loader.exec_module(mg)
    d = np.load(GOLDEN)
    spec = mg.spec()
    assert mg.initial_digest(spec.fields) == str(d["initial_sha256"])
    r = ctx.create(spec)
    r.write({k: d[f"spun_{k}"] for k in CARRIED})
    r.step(int(d["steps"]))
    got = r.read()
    errs = {k: rel_l2(got[k], d[f"final_{k}"], FLOOR.get(k, 0.0)) for k in CARRIED}
    rain = r.columns()["precipitation"]
    errs["precipitation"] = rel_l2(rain, d["final_precipitation"] - d["spun_precipitation"], 1e-6)
    print("golden:", ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    bad = {k: v for k, v in errs.items() if not v <= 1e-5}
    assert not bad, bad
    r.retire()
