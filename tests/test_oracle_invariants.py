"""Pins the oracle's whole step against the reference's invariant tests (src/core/invariants.test.ts).

The reference runs them with its own scenario presets; here they run on the benchmark configuration (analytic
Weisman-Klemp-type sounding, single-storm mode, ice microphysics, WENO transport, projection in stages) with the
oracle in faithful mode (FP32 field storage, as the reference's Float32Array fields). Thresholds are the reference's.
The same properties are checked on the device step in tests/test_gpu_invariants.py.
"""
import numpy as np
import pytest

import pyoracle as O
from parity import WATER, dual_divergence, level_mean, water_total
from meteolab_gb300.environment import Environment, SliderConfig
from meteolab_gb300.grid import GridOptions, create_grid
from meteolab_gb300.scenarios import RunSpec, Switches, baseline_profile, baseline_run, initial_fields

DT = 3.0


def small_grid(nx, ny):  # invariants.test.ts:6
    return create_grid(GridOptions(nx, ny, 24, nx * 1200.0, ny * 1125.0, 15_000.0))


def quiet_run(grid):
    """The sounding without a trigger: no bubble, no noise."""
    env = Environment(SliderConfig(), grid, baseline_profile())
    sw = Switches()
    return RunSpec(grid, env, sw, initial_fields(grid, env, 1, bubble=0.0, noise=0.0), 1, "quiet")


def storm_run(grid):
    return baseline_run(grid, seed=3, bubble=3.0, qv_max=0.016)


def total_water(m, spec):
    return water_total({k: m.get(k) for k in WATER}, m.get("precipitation"), spec)


@pytest.fixture(scope="module")
def background():
    grid = small_grid(12, 10)
    spec = quiet_run(grid)
    m = O.OracleModel(spec)
    m.step(DT, 3600)  # 3 hours
    return spec, m


def test_background_theta_stays_within_005_k_for_3_hours(background):  # :23
    spec, m = background
    th = m.get("theta")
    worst = max(abs(level_mean(th, spec.grid, z) - spec.env.theta[z]) for z in range(spec.grid.nz))
    assert worst < 0.05


def test_background_wind_stays_within_005_ms_for_3_hours(background):  # :24-28
    spec, m = background
    for name, env in (("u", spec.env.u), ("v", spec.env.v)):
        a = m.get(name)
        worst = max(abs(level_mean(a, spec.grid, z) - env[z]) for z in range(spec.grid.nz))
        assert worst < 0.05, name


def test_background_q_stays_within_1_percent_for_3_hours(background):  # :34
    spec, m = background
    q = m.get("q")
    worst = max(abs(level_mean(q, spec.grid, z) - spec.env.q[z]) for z in range(spec.grid.nz))
    assert worst / spec.env.q[0] < 0.01


def test_projection_removes_uniform_vertical_velocity():  # :40-47
    grid = small_grid(12, 10)
    rho = O.f64(quiet_run(grid).env.rho)
    u = np.zeros(grid.n, np.float32); v = np.zeros(grid.n, np.float32); w = np.zeros(grid.n, np.float32)
    w[grid.layer:(grid.nz - 1) * grid.layer] = 0.01
    cells = grid.layer * (grid.nz - 1)
    d0, d1, p = np.empty(cells), np.empty(cells), np.empty(cells)
    args, keep = O.grid_args(grid)
    O.lib().orc_pressure_project(*args, O.dp(rho), O.fp(u), O.fp(v), O.fp(w), 1.0, O.dp(d0), O.dp(d1), O.dp(p))
    for z in range(1, grid.nz - 1):
        assert abs(level_mean(w, grid, z)) < 1e-4


@pytest.fixture(scope="module")
def storm():
    grid = small_grid(20, 16)
    spec = storm_run(grid)
    m = O.OracleModel(spec)
    before = total_water(m, spec)
    m.step(DT, 300)  # 15 minutes
    return spec, m, before


def test_no_dual_cell_divergence_after_a_stormy_step(storm):  # :49-59
    spec, m, _ = storm
    div = dual_divergence(m.get("u"), m.get("v"), m.get("w"), spec.grid, spec.env.rho)
    assert np.max(np.abs(div)) < 1e-7
    assert m.counters()["clipped"] == 0


def test_water_is_conserved_within_001_percent_in_a_30_minute_storm_with_ice(storm):  # :84-94
    spec, m, before = storm
    m.step(DT, 300)  # to 30 minutes
    assert float(np.max(m.get("ice"))) > 1e-6
    assert float(np.max(m.get("graupel"))) > 1e-4
    assert abs(total_water(m, spec) / before - 1) < 1e-4


def test_numpy_gradient_and_divergence_restate_the_projection():
    """The FP64 operators the divergence checks use (parity.dual_divergence, parity.pressure_gradient) are the
    projection's own: applied to the oracle's pressure they leave the oracle's velocities divergence-free."""
    from parity import pressure_gradient
    grid = create_grid(GridOptions(16, 12, 20, 16 * 1200.0, 12 * 1125.0, 15_000.0, 100.0))
    rho = O.f64(quiet_run(grid).env.rho)
    rng = np.random.default_rng(5)
    u, v, w = ((rng.random(grid.n) - 0.5).astype(np.float32) * 10 for _ in range(3))
    w[:grid.layer] = 0; w[grid.n - grid.layer:] = 0
    u0, v0, w0 = u.copy(), v.copy(), w.copy()
    cells = grid.layer * (grid.nz - 1)
    d0, d1, p = np.empty(cells), np.empty(cells), np.empty(cells)
    args, keep = O.grid_args(grid)
    dt = 1.0
    O.lib().orc_pressure_project(*args, O.dp(rho), O.fp(u), O.fp(v), O.fp(w), dt, O.dp(d0), O.dp(d1), O.dp(p))
    gx, gy, gz = pressure_gradient(p, grid)
    div0 = dual_divergence(u0, v0, w0, grid, rho)
    div = dual_divergence(u0 - dt * gx, v0 - dt * gy, w0 - dt * gz, grid, rho)
    assert np.max(np.abs(div)) < 1e-10 * np.max(np.abs(div0))
