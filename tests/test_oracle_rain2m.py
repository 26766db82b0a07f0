"""The reference's two-moment rain tests (src/core/rain2m.test.ts) on the oracle (CPU): the drop-size bounds, the fall
speeds, rain from a deep cloud and its evaporation, the number's bookkeeping when ice takes or gives rain, the model
with the drop number carried and falling, and the breakup options. They pin the oracle's restatement of rain2m.ts
(oracle/oracle_rain2m.h) that the device's two-moment rain is checked against."""
import dataclasses
import math

import numpy as np

import pyoracle as O
from meteolab_gb300.environment import Environment, SliderConfig
from meteolab_gb300.grid import DEFAULT_GRID, create_grid
from meteolab_gb300.scenarios import RunSpec, Switches, initial_fields

DT = 3.0
RHO_W = 1000.0
XV_MIN, XV_MAX, RAIN_MIN = O.r2m_limits()


def close(a, b, digits):
    return abs(a - b) < 10 ** -digits / 2


def qsat(t, p):  # src/core/microphysics.ts:5
    return O.lib().orc_qsat(t, p)


def test_bounds_the_mean_drop_keeping_the_mass():  # rain2m.test.ts:8-19
    q, rho = 2e-3, 1.0
    few, many = O.r2m_bounded(q, 1, rho), O.r2m_bounded(q, 1e12, rho)
    assert close(q / (RHO_W * few), XV_MAX, 15) and close(q / (RHO_W * many), XV_MIN, 20)
    assert close(4 * O.r2m_dn(XV_MAX), 6e-3, 6)
    lam = (math.pi * RHO_W * 8e6 / (rho * q)) ** .25
    assert close(O.r2m_bounded(q, 0, rho), 8e6 / lam / rho, 0)
    assert O.r2m_bounded(0, 1e5, rho) == 0


def test_fall_speeds():  # :21-32
    rho = 1.1
    small, big = O.r2m_fall(1e-3, 1e6, rho), O.r2m_fall(1e-3, 1e3, rho)
    assert big[0] > small[0]
    for q, n in ((1e-3, 1e6), (1e-3, 1e4)):
        m, nn, z = O.r2m_fall(q, n, rho)
        assert z > m and m > nn and m < 11
    mp = O.r2m_fall(1e-3 / 1.2, O.r2m_bounded(1e-3 / 1.2, 0, 1.2), 1.2)[0]
    assert 4 < mp < 7.5


def test_rain_from_a_deep_cloud_and_its_evaporation():  # :34-53
    cell = np.array([.01356, 3e-3, 0, 0], np.float32)
    t = 0
    while t < 1800 and cell[2] < 1e-4:
        O.r2m_processes(cell, 290, 9e4, 1.07, DT)
        t += DT
    assert cell[2] > 1e-4 and t < 1500
    d = (6 * O.r2m_mean_volume(float(cell[2]), float(cell[3])) / math.pi) ** (1 / 3)
    assert 80e-6 < d < 1.5e-3
    dry = np.array([.004, 0, 1e-3, O.r2m_bounded(1e-3, 0, 1.1)], np.float32)
    mean0, total0 = float(dry[2]) / float(dry[3]), float(dry[0]) + float(dry[2])
    evap = O.r2m_processes(dry, 295, 9e4, 1.1, DT)
    assert evap > 0 and close(float(dry[0]) + float(dry[2]), total0, 9)
    ratio = float(dry[2]) / float(dry[3])
    assert ratio >= mean0 * (1 - 1e-6) and ratio < mean0 * 1.03


def test_number_follows_freezing_and_melting():  # :55-64
    cell = np.array([5e-4, 1e4], np.float32)
    O.r2m_number_change(cell, 1e-3, 1, 0)
    assert close(float(cell[1]), 5e3, 6)
    cell[0] = 1e-3
    O.r2m_number_change(cell, 5e-4, 1, 5e-4 / 2e3)
    assert close(float(cell[1]), 7e3, 3)
    cell[0] = RAIN_MIN / 2
    O.r2m_number_change(cell, 1e-3, 1, 0)
    assert cell[1] == 0


def test_runs_in_the_model():  # :66-78
    grid = create_grid(DEFAULT_GRID)
    env = Environment(SliderConfig(), grid)
    sw = Switches(rain_moments=2)
    fields = initial_fields(grid, env, 3, bubble=0.0, noise=0.0)
    fields["rainNumber"] = np.zeros(grid.n)
    layer = grid.layer
    for z in range(grid.nz):
        if 2000 < grid.zs[z] < 4000:
            for c in range(6):
                i = c + z * layer
                fields["rain"][i] = 2e-3
                fields["rainNumber"][i] = np.float32(O.r2m_bounded(2e-3, 0, env.rho[z]))
    m = O.OracleModel(RunSpec(grid, env, sw, fields, 3, "shaft"))
    m.step(DT, 200)
    assert float(np.sum(m.get("precipitation"))) > 0
    rain, num = m.get("rain"), m.get("rainNumber")
    assert (num >= 0).all()
    wet = rain > 1e-7
    xv = rain[wet] / (RHO_W * num[wet])
    assert (xv >= XV_MIN * .999).all() and (xv <= XV_MAX * 1.001).all()


def test_breakup_only_with_the_switch():  # :80-91
    def settle(b):
        tk, p = 288, 9e4
        rho = p / (287 * tk)
        cell = np.array([qsat(tk - 273.15, p) * 1.0001, 0, 2e-3, 2e-3 / (RHO_W * math.pi * 1.2e-3 ** 3)], np.float32)
        t = 0
        while t < 1800:
            cell[1] = 0
            O.r2m_processes(cell, tk, p, rho, DT, b)
            t += DT
        assert close(float(cell[2]), 2e-3, 6)
        return O.r2m_dn(O.r2m_mean_volume(float(cell[2]), float(cell[3]))) * 1000
    assert close(settle("none"), 1.2, 2)
    assert close(settle("morrison"), .6, 1)
    v = settle("nssl")
    assert .65 < v < .8
