"""The reference's two-moment graupel and hail tests (src/core/ice2m.test.ts) on the oracle (CPU): the gamma functions
and the fall-speed table, the density from the volume and the bounded mean particle, the moment-weighted fall speeds,
the largest stones from the tail, riming, densification and melting, Bigg freezing, the model with both two-moment
classes carried and falling, and the charging by a class's own moments. They pin the oracle's restatement of ice2m.ts
(oracle/oracle_ice2m.h) that the device's two-moment graupel and hail are checked against. (The radar case of that
file, :92-98, concerns src/core/radar.ts, which is not on the model step.)"""
import math

import numpy as np

import pyoracle as O
from meteolab_gb300.environment import Environment, SliderConfig
from meteolab_gb300.grid import DEFAULT_GRID, create_grid
from meteolab_gb300.scenarios import RunSpec, Switches, initial_fields

DT = 3.0


def close(a, b, digits):  # vitest toBeCloseTo
    return abs(a - b) < 10 ** -digits / 2


def test_mathematics():  # ice2m.test.ts:15-19
    assert close(O.i2m_gamma(5), 24, 10) and close(O.i2m_gamma(.5), math.sqrt(math.pi), 10) and close(O.i2m_gamma(2.9), 1.8273551, 6)
    assert close(O.i2m_upper_gamma(1, 2), math.exp(-2), 12) and close(O.i2m_upper_gamma(2, 1), 2 * math.exp(-1), 12)
    assert O.i2m_upper_gamma(4, 0) == 1
    assert O.i2m_fall_law(450) == (145.26, .60572)
    assert O.i2m_fall_law(900)[0] > 189 and close(O.i2m_fall_law(100)[0], (62.923 + 94.122) / 2, 3)


def test_density_from_the_volume_and_the_bounded_mean_particle():  # :21-28
    assert close(O.i2m_density("graupel", 1e-3, 1e-3 / 400), 400, 3)
    assert O.i2m_density("graupel", 1e-3, 1) == 170 and O.i2m_density("hail", 1e-3, 1) == 500 and O.i2m_density("hail", 1e-3, 0) == 800
    n = O.i2m_bounded("graupel", 1e-3, 1e-3, 1e-3 / 500)
    xv = 1e-3 / (500 * n)
    assert close(4 * (6 * xv / math.pi) ** (1 / 3) / 6 ** (1 / 3), 20e-3, 6)


def test_fall_speeds():  # :30-36
    light, dense = O.i2m_moment_speed("graupel", 1e-3, 1e3, 1e-3 / 200, 1, 3), O.i2m_moment_speed("graupel", 1e-3, 1e3, 1e-3 / 800, 1, 3)
    assert dense > light
    z, m, nn = (O.i2m_moment_speed("hail", 2e-3, 100, 2e-3 / 900, 1, k) for k in (6, 3, 0))
    assert z > m > nn and 10 < m < 45


def test_largest_stones_from_the_tail():  # :38-41
    many, few = O.i2m_largest("hail", 2e-3, 1e4, 2e-3 / 900, 1), O.i2m_largest("hail", 2e-3, 10, 2e-3 / 900, 1)
    assert few > many and few > 20e-3 and many < 15e-3


def test_rimes_densifies_and_melts():  # :43-56
    exner, p, rho = .8, 6e4, .8
    f = O.i2m_node(theta=263.15 / exner, q=2.6e-3, cloud=2e-3, graupel=1e-3, graupelNumber=1e4, graupelVolume=1e-3 / 300)
    ix = {k: j for j, k in enumerate(O.I2M_ORDER)}
    water = float(f[ix["cloud"]]) + float(f[ix["graupel"]]) + float(f[ix["q"]])
    for _ in range(20):
        O.i2m_processes(f, exner, p, rho, DT)
    assert f[ix["graupel"]] > 1e-3 and f[ix["cloud"]] < 2e-3
    assert close(float(f[ix["cloud"]]) + float(f[ix["graupel"]]) + float(f[ix["q"]]) + float(f[ix["rain"]]), water, 8)
    assert f[ix["graupel"]] / f[ix["graupelVolume"]] > 300
    warm = O.i2m_node(theta=283.15 / .95, q=5e-3, graupel=2e-3, graupelNumber=2e3, graupelVolume=2e-3 / 600)
    cooling, _, _ = O.i2m_processes(warm, .95, 9e4, 1.1, DT)
    assert cooling > 0 and warm[ix["rain"]] > 0 and warm[ix["rainNumber"]] > 0
    assert close(float(warm[ix["rain"]]) + float(warm[ix["graupel"]]), 2e-3, 8)


def test_bigg_freezing():  # :58-64
    f = O.i2m_node(theta=253.15 / .7, q=1e-3, rain=1e-3, rainNumber=O.r2m_bounded(1e-3, 0, .7))
    ix = {k: j for j, k in enumerate(O.I2M_ORDER)}
    O.i2m_processes(f, .7, 5e4, .7, DT)
    assert f[ix["graupel"]] > 0 and f[ix["graupelNumber"]] > 0
    assert close(float(f[ix["graupel"]]) + float(f[ix["rain"]]) + float(f[ix["q"]]), 2e-3, 8)


def shafts(seed=5):
    """:66-70: a summer day with graupel (2 g/kg, 2000 per kg at 500 kg/m3) and hail (1 g/kg, 50 per kg at 900 kg/m3)
    from 3 to 7 km over eight columns, two-moment rain and ice."""
    grid = create_grid(DEFAULT_GRID)
    env = Environment(SliderConfig(), grid)
    fields = initial_fields(grid, env, seed)
    for k in ("rainNumber",) + O.ICE2M:
        fields[k] = np.zeros(grid.n)
    for z in range(grid.nz):
        if 3000 < grid.zs[z] < 7000:
            for c in range(8):
                i = c + z * grid.layer
                fields["graupel"][i], fields["graupelNumber"][i], fields["graupelVolume"][i] = 2e-3, 2e3, 2e-3 / 500
                fields["hail"][i], fields["hailNumber"][i], fields["hailVolume"][i] = 1e-3, 50, 1e-3 / 900
    return RunSpec(grid, env, Switches(rain_moments=2, ice_moments=2), fields, seed, "ice2m-shafts")


def test_runs_in_the_model():  # :66-80
    m = O.OracleModel(shafts())
    m.step(DT, 120)
    assert float(np.sum(m.get("precipitation"))) > 0
    for q, n, v in (("graupel", "graupelNumber", "graupelVolume"), ("hail", "hailNumber", "hailVolume")):
        qa, na, va = m.get(q), m.get(n), m.get(v)
        assert np.isfinite(na).all() and (na >= 0).all()
        big = qa > 1e-7
        assert (na[big] > 0).all()
        d = qa[big] / va[big]
        assert (d > 160).all() and (d < 910).all()


def test_charges_by_the_moments_as_by_the_fixed_intercept():  # :100-108
    rho, q = .7, 2e-3
    lam = (math.pi * 400 * 4e4 / (rho * q)) ** .25
    n = 4e4 / lam / rho
    one = O.charging_rate_2m(-15, rho, 1e-3, 1e-4, 2e-4, q, 0, 1, False, False, 1e5)
    two = O.charging_rate_2m(-15, rho, 1e-3, 1e-4, 2e-4, q, 0, 1, False, False, 1e5,
                             (O.i2m_rimer_moments("graupel", q, n, q / 400, rho), None))
    assert one != 0 and math.copysign(1, two) == math.copysign(1, one) and .2 < abs(two / one) < 5


def test_charging_without_moments_is_the_one_moment_rate():
    """A missing entry (a class below 1e-9 kg/kg or without particles: rimerMoments null) takes the fixed intercept's
    moments, as `twoMoment?.[j] ?? exponentialMoments(...)` does (charge.ts:153-155)."""
    args = (-15, .7, 1e-3, 1e-4, 2e-4, 2e-3, 1e-3, 1, False, False, 1e5)
    assert O.charging_rate_2m(*args) == O.charging_rate_2m(*args, (None, None))
    assert O.i2m_rimer_moments("graupel", 1e-10, 10, 1e-13, .7) is None and O.i2m_rimer_moments("hail", 1e-3, 0, 1e-6, .7) is None
