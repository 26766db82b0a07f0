"""The host set-up's base state and parcels against the reference's environment tests (src/core/environment.test.ts),
read as known answers: the slider profile's wind nodes (:5-33), its neutralising warmth (:35-58, the explicit cases and
the «Летний день» scenario), and the night inversion (:60-80). The scenario values are the reference's
(src/core/fixtures.ts:6-12 SUMMER_DAY; src/core/scenarios.ts:29-36 SUMMER_AIR, LIGHT_WIND, and the two scenarios'
own values at :55 and :94)."""
import dataclasses

import pytest

from conftest import close
from meteolab_gb300.environment import NIGHT_DEPTH, Environment, SliderConfig
from meteolab_gb300.grid import DEFAULT_GRID, create_grid
from meteolab_gb300.sounding import lift_parcel

GRID = create_grid(DEFAULT_GRID)
SUMMER_AIR = dict(surfaceTemp=28, rhSurface=55, rhLow=50, rhMid=45, rhUpper=30, lapseLow=9.3, lapseMid=6.3, lapseUpper=6.5,
                  capStrength=1, capHeight=1.4, moistLayer=1)
LIGHT_WIND = dict(wind0=2, wind3=5, wind6=9, wind10=14, windDir0=200, windDir3=230, windDir6=250, windDir10=260)


def env(**values):
    return Environment(SliderConfig(**values), GRID)


# ---- wind profile (environment.test.ts:5-33)
def test_the_wind_turns_across_north_along_the_shorter_arc():
    assert close(env(windDir0=350, windDir3=10).wind_direction(1500), 0, 9)
    assert close(env(windDir0=10, windDir3=350).wind_direction(750), 5, 9)
    assert close(env(windDir0=300, windDir3=60).wind_direction(1500), 0, 9)
    u, v = env(windDir0=350, windDir3=10).wind_uv(1500)
    assert v < 0 and abs(u) < 1e-9


def test_the_wind_passes_the_optional_half_and_one_km_nodes():
    e = env(wind0=5, windDir0=120, wind05=10, windDir05=150, wind1=14, windDir1=180, wind3=20, windDir3=240)
    assert e.wind_scalar(500) == 10 and e.wind_direction(1000) == 180
    assert close(e.wind_scalar(750), 12, 9) and close(e.wind_direction(2000), 210, 9)
    assert close(env(wind0=5, windDir0=120, wind3=20, windDir3=240).wind_scalar(1500), 12.5, 9)


def test_profiles_that_do_not_cross_north_are_unchanged():
    assert env(windDir0=160, windDir3=185).wind_direction(1500) == 172.5
    assert env(windDir0=140, windDir3=200).wind_direction(3000) == 200


# ---- slider profiles are not unstable by themselves (environment.test.ts:35-58)
def worst_thv_lapse(**values):
    e = env(**values)
    thv = lambda z: e.theta_env(z) * (1 + .61 * e.q_env(z))
    return min(0.0, min((thv(z + 25) - thv(z)) / .025 for z in range(0, 14_000, 25)))


def test_the_steepest_slider_settings_are_neutralised():
    assert worst_thv_lapse(lapseLow=11, rhSurface=90, rhLow=20, capStrength=6, capHeight=.5, moistLayer=2.5) > -.5
    assert worst_thv_lapse(lapseLow=9.8, capStrength=4, capHeight=2, moistLayer=1.5, nightInversion=8) > -.5


def test_summer_day_is_warmed_only_where_needed_and_keeps_its_cape():
    values = dict(SUMMER_AIR, **LIGHT_WIND)
    assert worst_thv_lapse(**values) > -.5
    e = env(**values)
    assert close(e.temperature_env(500), 28 - 9.3 * .5, 6)
    assert abs(lift_parcel(e, GRID.height, "ml").cape / 2721 - 1) < .05  # the plain profile's ML CAPE, 2721 J/kg


# ---- night inversion (environment.test.ts:60-80)
def test_the_night_cools_the_ground_the_residual_layer_and_nothing_above_the_lid():
    day, dawn = env(moistLayer=1), env(moistLayer=1, nightInversion=6)
    assert close(day.temperature_env(0) - dawn.temperature_env(0), 6, 6)
    assert close(dawn.night_deficit(NIGHT_DEPTH), 1.5, 6)
    assert close(dawn.night_deficit(1200), 1.5, 6)
    assert dawn.night_deficit(3000) == 0 and day.night_deficit(0) == 0


def test_the_dawn_inversion_is_moist_unsaturated_and_caps_the_surface_parcel():
    values = dict(SUMMER_AIR, **LIGHT_WIND)
    values.update(capStrength=0, moistLayer=0, nightInversion=6)
    morning = env(**values)
    t = morning.temperature_env(0)
    td = morning.dewpoint(morning.q_env(0), 0)
    assert td < t and t - td < 6
    assert lift_parcel(morning, GRID.height, "sb").cin > 100
    values["nightInversion"] = 0
    assert lift_parcel(env(**values), GRID.height, "sb").cin < 10


def test_regime_grid_points_span_the_cape_and_shear_levels():
    """The uneven batch's regime points (scenarios.regime_runs): the lid-free points' mixed-layer CAPE within 10 % of
    their row's level (500-4000 J/kg, set through the moisture / lapse-rate knob), the shear exactly the column's
    level, lids of 0-4 K at 1.5-3 km, and a lid never raising the CAPE."""
    from meteolab_gb300.grid import LARGE_GRID
    from meteolab_gb300.scenarios import CAPE_LEVELS, SHEAR_LEVELS, regime_runs
    runs = regime_runs(GRID, create_grid(LARGE_GRID), n_small=10, n_large=2)
    assert len(runs) == 12 and sum(r.grid.nx == 80 for r in runs) == 2
    for r in runs:
        m = r.meta
        i, j = (int(x) for x in r.label.replace("cape", "").split("-shear"))
        assert m["cape_level"] == CAPE_LEVELS[i]
        assert abs(m["shear"] - SHEAR_LEVELS[j]) < 1e-9 * max(1.0, SHEAR_LEVELS[j])
        if m["lid_k"] == 0:
            assert abs(m["cape"] / m["cape_level"] - 1) < .1, (r.label, m)
        else:
            assert 0 < m["lid_k"] <= 4 and 1.5 <= m["lid_km"] <= 3
            assert m["cape"] <= m["cape_level"] * 1.1
