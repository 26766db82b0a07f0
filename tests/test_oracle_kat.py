"""Pins the oracle against the reference's own known-answer tests for the step.

Each test restates one of the reference's unit tests (vitest, src/core/*.test.ts) with its inputs and tolerances,
run against the oracle (oracle/pyoracle.py). The reference ships no stored golden field vectors for the step; these
tests plus the invariant tests in test_oracle_invariants.py are what pins the oracle.
"""
import math

import numpy as np
import pytest

import pyoracle as O
from conftest import close
from meteolab_gb300.grid import DEFAULT_GRID, GridOptions, create_grid, level_at

CP, LV, KAPPA, LF, LS = 1004.0, 2.5e6, 0.286, 3.34e5, 2.5e6 + 3.34e5
L = O.lib()


def f32(x):
    return float(np.float32(x))


# ------------------------------------------------------------------ src/core/advection.test.ts
def test_weno_reconstructs_smooth_data_and_does_not_overshoot():  # :5-11
    avg = lambda i: i * i + 1 / 12
    assert close(L.orc_weno(avg(-2), avg(-1), avg(0), avg(1), avg(2)), 0.25, 3)
    step = L.orc_weno(0, 0, 0, 1, 1)
    assert -1e-9 <= step <= 1


def _transport(grid, rho, u, v, w, q, dt, steps, monotone=True):
    args, keep = O.grid_args(grid)
    rho = O.f64(rho)
    L.orc_transport(*args, O.dp(rho), O.fp(u), O.fp(v), O.fp(w), O.fp(q), dt, steps, 1 if monotone else 0,
                    None, None, None, None)
    return q


def test_transport_keeps_uniform_field_and_conserves_mass():  # :21-30
    grid = create_grid(GridOptions(20, 6, 5, 20 * 1000.0, 6000.0, 4000.0))
    rho = [1.2, 1.1, 1, 0.9, 0.8]
    u = np.full(grid.n, 10, np.float32); v = np.zeros(grid.n, np.float32); w = np.zeros(grid.n, np.float32)
    q = np.full(grid.n, 0.01, np.float32)
    _transport(grid, rho, u, v, w, q, 5, 100)
    assert np.max(np.abs(q.astype(np.float64) - 0.01)) < 1e-8
    i = np.arange(grid.n)
    blob = np.exp(-((((i % 20) - 10) / 2) ** 2)).astype(np.float32)
    mass = lambda a: float(np.sum(a.astype(np.float64) * np.array(rho)[i // grid.layer]))
    before = mass(blob)
    _transport(grid, rho, u, v, w, blob, 5, 100)
    assert abs(mass(blob) / before - 1) < 1e-5


def test_transport_projects_random_faces_to_zero_divergence():  # :32-46
    grid = create_grid(GridOptions(12, 10, 8, 12000.0, 10000.0, 7000.0))
    rho = [1.2, 1.1, 1, 0.9, 0.8, 0.7, 0.6, 0.5]
    rng = np.random.default_rng(7)
    rnd = lambda: (20 * (rng.random(grid.n) - 0.5)).astype(np.float32)
    u, v, w = rnd(), rnd(), rnd()
    w[:grid.layer] = 0; w[grid.n - grid.layer:] = 0
    uniform = np.full(grid.n, 0.01, np.float32)
    _transport(grid, rho, u, v, w, uniform, 5, 50)
    assert np.max(np.abs(uniform.astype(np.float64) - 0.01)) < 1e-7
    i = np.arange(grid.n); z = i // grid.layer
    weight = np.array(rho)[z] * np.where((z == 0) | (z == grid.nz - 1), 0.5, 1.0)
    blob = np.exp(-(((i % 12) - 6) ** 2 + (((i // 12) % 10) - 5) ** 2) / 4).astype(np.float32)
    before = float(np.sum(blob * weight))
    _transport(grid, rho, u, v, w, blob, 5, 50)
    assert abs(float(np.sum(blob.astype(np.float64) * weight)) / before - 1) < 1e-6


def test_transport_skips_empty_rows_exactly():  # :48-65
    grid = create_grid(GridOptions(16, 12, 10, 16000.0, 12000.0, 9000.0))
    rho = [1.2 - 0.07 * z for z in range(10)]
    rng = np.random.default_rng(11)
    rnd = lambda: (20 * (rng.random(grid.n) - 0.5)).astype(np.float32)
    u, v, w = rnd(), rnd(), rnd()
    w[:grid.layer] = 0; w[grid.n - grid.layer:] = 0
    i = np.arange(grid.n); x, y, z = i % 16, (i // 16) % 12, i // 192
    inside = (np.abs(x - 4) <= 1) & (np.abs(y - 3) <= 1) & (np.abs(z - 4) <= 1)
    sparse = np.where(inside, 1e-3, 0).astype(np.float32)
    dense = np.where(inside, 1e-3, 1e-30).astype(np.float32)
    for _ in range(3):
        _transport(grid, rho, u, v, w, sparse, 5, 1)
        _transport(grid, rho, u, v, w, dense, 5, 1)
    assert np.max(np.abs(sparse.astype(np.float64) - dense)) < 1e-12


@pytest.mark.slow
def test_transport_carries_blob_around_domain():  # :67-74
    grid = create_grid(GridOptions(40, 6, 5, 40 * 1000.0, 6000.0, 4000.0))
    rho = [1.2, 1.1, 1, 0.9, 0.8]
    u = np.full(grid.n, 10, np.float32); v = np.zeros(grid.n, np.float32); w = np.zeros(grid.n, np.float32)
    i = np.arange(grid.n)
    q = np.exp(-((((i % 40) - 20) / 3) ** 2)).astype(np.float32)
    _transport(grid, rho, u, v, w, q, 1, 4000)
    assert q.max() > 0.88 and q.min() > -0.02
    assert int(np.argmax(q)) % 40 == 20


# ------------------------------------------------------------------ src/core/microphysics.test.ts
def test_rain_fall_speed():  # :7-13
    assert close(L.orc_fall_speed(0.001, 1.2, 1.2), 5.68, 1)
    assert close(L.orc_fall_speed(0.005, 1.2, 1.2), 7.05, 1)
    assert close(L.orc_fall_speed(0.001, 0.6, 1.2) / L.orc_fall_speed(0.001, 1.2, 1.2), 0.5 ** 0.1364 * math.sqrt(2), 6)
    assert L.orc_fall_speed(0, 1.2, 1.2) == 0


def test_autoconversion_and_accretion():  # :15-23
    _, c = O.cell("rain", dict(q=0.01, cloud=0.003, rain=0), p=80000, rho=1, dt=1, aux=280)
    assert close(c["rain"], 0.001 * 0.002, 8)
    _, c = O.cell("rain", dict(q=0.01, cloud=0.002, rain=0.002), p=80000, rho=1, dt=1, aux=280)
    assert close(c["rain"] - f32(0.002), 0.001 * 0.001 + 2.2 * 0.002 * 0.002 ** 0.875, 8)
    assert close(float(c["cloud"]) + float(c["rain"]), 0.004, 8)


def test_rain_evaporation():  # :25-35
    p, tk = 85000.0, 290.0
    qs = L.orc_qsat(tk - 273.15, p)
    evap, c = O.cell("rain", dict(q=0.5 * qs, rain=0.001), p=p, rho=1, dt=1, aux=tk)
    assert 0.002 < evap / 0.001 < 0.01
    assert close(float(c["q"]) + float(c["rain"]), f32(0.5 * qs) + f32(0.001), 8)
    _, c = O.cell("rain", dict(q=0.999 * qs, rain=0.01), p=p, rho=1, dt=1000, aux=tk)
    assert c["q"] <= qs
    evap, _ = O.cell("rain", dict(q=1.1 * qs, rain=0.001), p=p, rho=1, dt=1, aux=tk)
    assert evap == 0


def _sat_cell(temp_c, q, cloud, p=70000.0):
    exner = (p / 100000) ** KAPPA
    return dict(theta=(temp_c + 273.15) / exner, q=q, cloud=cloud), exner


def test_saturation_adjustment():  # :38-72
    p = 70000.0
    cell0, exner = _sat_cell(10, 1.3 * L.orc_qsat(10, p), 0)
    thL = lambda c: float(c["theta"]) - LV / (CP * exner) * float(c["cloud"])
    qs_of = lambda c: L.orc_qsat(float(c["theta"]) * exner - 273.15, p)
    c0 = {k: f32(v) for k, v in cell0.items()}
    water, th_l = c0["q"] + c0["cloud"], thL(c0)
    cond, c = O.cell("satadjust", cell0, exner=exner, p=p)
    assert cond > 0
    assert abs(float(c["q"]) / qs_of(c) - 1) < 1e-4
    assert c["cloud"] < 0.3 * L.orc_qsat(10, p)
    assert close(float(c["q"]) + float(c["cloud"]), water, 9)
    assert close(thL(c), th_l, 3)
    partial, _ = _sat_cell(10, 0.95 * L.orc_qsat(10, p), 0.005)
    _, c = O.cell("satadjust", partial, exner=exner, p=p)
    assert abs(float(c["q"]) / qs_of(c) - 1) < 1e-4 and c["cloud"] > 0
    gone, _ = _sat_cell(10, 0.5 * L.orc_qsat(10, p), 0.0005)
    g0 = {k: f32(v) for k, v in gone.items()}
    cond, c = O.cell("satadjust", gone, exner=exner, p=p)
    assert close(cond, -0.0005, 9) and c["cloud"] == 0 and c["q"] < qs_of(c)
    assert close(thL(c), thL(g0), 3)
    clear, _ = _sat_cell(10, 0.7 * L.orc_qsat(10, p), 0)
    cl0 = {k: f32(v) for k, v in clear.items()}
    cond, c = O.cell("satadjust", clear, exner=exner, p=p)
    assert cond == 0 and c["theta"] == cl0["theta"] and c["q"] == cl0["q"]


# ------------------------------------------------------------------ src/core/ice.test.ts
def test_ice_saturation_and_nucleation():  # :9-17
    assert close(L.orc_qsat_ice(-20, 50000) / L.orc_qsat(-20, 50000), 0.82, 2)
    assert close(L.orc_qsat_ice(-1e-9, 80000) / L.orc_qsat(0, 80000), 1, 3)
    assert L.orc_cooper(-3) == 0
    assert close(L.orc_cooper(-20) / 1e3, 2.2, 1)
    assert L.orc_cooper(-60) == 250e3


def test_secondary_ice():  # :19-25
    assert close(L.orc_splintering(-5) * 3.5e8 * 1e-6, 350, 6)
    assert L.orc_splintering(-2) == 0 and L.orc_splintering(-9) == 0
    assert close(L.orc_splintering(-4), 0.5, 9) and close(L.orc_splintering(-6.5), 0.5, 9)
    per_drop = L.orc_fragments(2000) * 1000 * math.pi / 6 * (7 / 2000) ** 3
    assert close(per_drop, 2.5e13 * (7 / 2000) ** 4, 0)


def test_crystal_growth_habits():  # :27-34
    m = 1e-10
    k = L.orc_koenig
    assert k(-15, m) > 4 * k(-9, m) and k(-5, m) > 1.5 * k(-9, m)
    assert k(-15.5, m) < k(-15, m) and k(-40, m) == k(-31, m)
    assert 0.5 < k(-15, m) * 60 / m < 5
    assert close(L.orc_plate_size(m) * 1e6, 103, -1)
    assert L.orc_plate_size(m) > 1.5 * L.orc_crystal_size(m, 1, 1)


def test_snow_falls_about_one_metre_per_second():  # :36-39
    v = L.orc_snow_fall_speed(1e-3 / 1.1, 1.1, 1.1)
    assert 0.8 < v < 1.5


def test_cloud_water_stays_liquid_to_minus_38():  # :41-48
    p = 40000.0; exner = (p / 1e5) ** KAPPA
    v0 = dict(theta=243.15 / exner, q=1.2 * L.orc_qsat(-30, p), cloud=0, ice=1e-5)
    total = f32(v0["q"]) + f32(v0["cloud"]) + f32(v0["ice"])
    _, c = O.cell("satmixed", v0, exner=exner, p=p)
    assert close(float(c["q"]) + float(c["cloud"]) + float(c["ice"]), total, 9)
    assert c["cloud"] > 0 and c["ice"] == np.float32(1e-5)
    assert close(float(c["q"]) / L.orc_qsat(float(c["theta"]) * exner - 273.15, p), 1, 3)


def test_droplets_freeze_below_minus_38():  # :50-57
    p = 25000.0; exner = (p / 1e5) ** KAPPA
    v0 = dict(theta=228.15 / exner, q=L.orc_qsat(-45, p), cloud=5e-4, ice=0)
    total, before = f32(v0["q"]) + f32(v0["cloud"]), f32(v0["theta"])
    _, c = O.cell("satmixed", v0, exner=exner, p=p)
    assert c["cloud"] == 0 and close(float(c["q"]) + float(c["ice"]), total, 9)
    assert close(float(c["q"]) / L.orc_qsat_ice(float(c["theta"]) * exner - 273.15, p), 1, 3)
    assert close((float(c["theta"]) - before) * exner, (LF * 5e-4 + LS * (float(c["ice"]) - 5e-4)) / CP, 3)


def test_ice_melts_above_zero():  # :59-64
    p = 80000.0; exner = (p / 1e5) ** KAPPA
    _, c = O.cell("satmixed", dict(theta=275.15 / exner, q=L.orc_qsat(2, p), cloud=0, ice=1e-3), exner=exner, p=p)
    assert c["ice"] == 0 and c["cloud"] > 9e-4 and float(c["theta"]) * exner < 275.15


def test_rain_freezes_below_minus_38():  # :66-70
    exner = (25000 / 1e5) ** KAPPA
    v0 = dict(theta=230 / exner, rain=1e-3, graupel=0)
    _, c = O.cell("freeze", v0, exner=exner)
    assert c["rain"] == 0 and close(c["graupel"], 1e-3, 9)
    assert close((float(c["theta"]) - f32(230 / exner)) * exner, LF / CP * 1e-3, 5)


def _iterate(which, state, n, **kw):
    names = ("theta", "q", "cloud", "ice", "snow", "rain", "graupel", "hail", "number")
    v = np.array([state.get(k, 0.0) for k in names], dtype=np.float32)
    code = {"ice": 4, "satmixed": 2, "snow": 5, "graupel": 6, "hail": 7}
    out = 0.0
    for _ in range(n):
        for w in which:
            out = L.orc_cell(code[w], O.fp(v), kw["exner"], kw["p"], kw.get("rho", 1), kw.get("dt", 1), kw.get("aux", 0))
    return out, {k: v[i] for i, k in enumerate(names)}


def test_bergeron_growth_conserves_water():  # :72-84
    p = 50000.0; exner = (p / 1e5) ** KAPPA; rho = 0.7
    s = dict(theta=253.15 / exner, q=L.orc_qsat(-20, p), cloud=1e-3, ice=0, snow=0, number=0)
    water = lambda c: float(c["q"]) + float(c["cloud"]) + float(c["ice"]) + float(c["snow"])
    before = f32(s["q"]) + f32(s["cloud"])
    _, c = _iterate(["ice"], s, 1, exner=exner, p=p, rho=rho, dt=1)
    assert L.orc_cooper(-20) * 1e-12 / rho < c["ice"] < 2 * L.orc_cooper(-20) * 1e-12 / rho
    names = ("theta", "q", "cloud", "ice", "snow", "rain", "graupel", "hail", "number")
    v = np.array([c[k] for k in names], dtype=np.float32)
    for _ in range(600):
        L.orc_cell(4, O.fp(v), exner, p, rho, 1, 0)
        L.orc_cell(2, O.fp(v), exner, p, rho, 1, 0)
    c = {k: v[i] for i, k in enumerate(names)}
    assert float(c["ice"]) + float(c["snow"]) > 1e-6 and c["cloud"] < 1e-3
    assert close(water(c), before, 7)
    assert c["cloud"] > 5e-4


def test_ice_sublimates_in_dry_air():  # :86-90
    p = 30000.0; exner = (p / 1e5) ** KAPPA
    cool, c = O.cell("ice", dict(theta=243.15 / exner, q=0.5 * L.orc_qsat_ice(-30, p), ice=1e-4, snow=0, number=1e-4 / 1e-11),
                     exner=exner, p=p, rho=0.45, dt=10)
    assert c["ice"] < np.float32(1e-4) and cool > 0 and c["number"] < np.float32(1e-4 / 1e-11)


def test_snow_grows_and_melts():  # :92-105
    p = 60000.0; exner = (p / 1e5) ** KAPPA; rho = 0.8
    cold = dict(theta=258.15 / exner, q=L.orc_qsat(-15, p), cloud=5e-4, ice=2e-3, snow=1e-3, rain=0)
    water = lambda c: sum(float(c[k]) for k in ("q", "cloud", "ice", "snow", "rain"))
    before = sum(f32(cold[k]) for k in ("q", "cloud", "ice", "snow", "rain"))
    _, c = _iterate(["snow"], cold, 60, exner=exner, p=p, rho=rho, dt=1, aux=1.1)
    assert c["snow"] > 1e-3
    assert abs(water(c) - before) < 2e-9
    warm = dict(theta=278.15 / exner, q=0.005, cloud=0, ice=0, snow=1e-3, rain=0)
    cool, c = O.cell("snow", warm, exner=exner, p=p, rho=rho, dt=10, aux=1.1)
    assert c["rain"] > 0 and close(float(c["rain"]) + float(c["snow"]), 1e-3, 9)
    assert close(cool * exner, LF / CP * float(c["rain"]), 5)


# ------------------------------------------------------------------ src/core/graupel.test.ts
def _g_cell(tk, p, **v):
    exner = (p / 1e5) ** KAPPA
    d = dict(theta=tk / exner); d.update(v)
    return d, exner


def test_graupel_falls_five_to_ten():  # :14-17
    v = L.orc_graupel_fall_speed(1e-3 / 1.1, 1.1)
    assert 5 < v < 10


def test_graupel_freezes_rain_faster_when_colder():  # :19-26
    def frozen_after(tk):
        c0, ex = _g_cell(tk, 50000, rain=2e-3)
        _, c = O.cell("graupel", c0, exner=ex, p=50000, rho=0.7, dt=10)
        return float(c["graupel"])
    assert frozen_after(253.15) > 100 * frozen_after(268.15)
    c0, ex = _g_cell(253.15, 50000, q=1.5e-3, rain=2e-3)
    _, c = O.cell("graupel", c0, exner=ex, p=50000, rho=0.7, dt=10)
    assert close((float(c["theta"]) - f32(c0["theta"])) * ex, LF / CP * float(c["graupel"]), 5)


def test_graupel_rimes_and_melts():  # :28-39
    c0, ex = _g_cell(263.15, 60000, q=1e-3, cloud=2e-3, snow=1e-3, graupel=2e-3)
    water = lambda c: sum(float(c[k]) for k in ("q", "cloud", "ice", "snow", "rain", "graupel"))
    before = sum(f32(c0.get(k, 0)) for k in ("q", "cloud", "ice", "snow", "rain", "graupel"))
    _, c = _iterate(["graupel"], c0, 30, exner=ex, p=60000, rho=0.8, dt=1)
    assert c["cloud"] < 2e-3 and c["graupel"] > 2e-3 and close(water(c), before, 9)
    w0, ex = _g_cell(281.15, 80000, q=5e-3, graupel=2e-3)
    cool, c = O.cell("graupel", w0, exner=ex, p=80000, rho=1, dt=10)
    assert c["rain"] > 0 and close(float(c["rain"]) + float(c["graupel"]), 2e-3, 9)
    assert close(cool * ex, LF / CP * float(c["rain"]), 5)


# ------------------------------------------------------------------ src/core/hail.test.ts
def test_hail_fall_speed_and_size():  # :17-28
    v = L.orc_hail_fall_speed(1e-3 / 1.1, 1.1)
    assert 10 < v < 16 and v > 1.3 * L.orc_graupel_fall_speed(1e-3 / 1.1, 1.1)
    d2, d10 = L.orc_hail_max_diameter(2e-3 / 1.1, 1.1), L.orc_hail_max_diameter(1e-2 / 1.1, 1.1)
    assert d2 > 0.01 and d10 < 0.03 and d10 > d2 and L.orc_hail_max_diameter(0, 1.1) == 0


def test_hail_born_in_wet_growth():  # :30-39
    species = ("q", "cloud", "ice", "snow", "rain", "graupel", "hail")
    water = lambda c: sum(float(c[k]) for k in species)
    c0, ex = _g_cell(265.15, 55000, q=4e-3, cloud=4e-3, rain=4e-3, graupel=4e-3)
    before = sum(f32(c0.get(k, 0)) for k in species)
    _, c = _iterate(["hail"], c0, 60, exner=ex, p=55000, rho=0.75, dt=1)
    assert c["hail"] > 1e-3 and close(water(c), before, 8)
    d0, ex = _g_cell(243.15, 35000, q=3e-4, cloud=2e-4, graupel=2e-3)
    _, c = _iterate(["hail"], d0, 60, exner=ex, p=35000, rho=0.5, dt=1)
    assert c["hail"] == 0


def test_hail_wet_growth_limit():  # :41-53
    species = ("q", "cloud", "ice", "snow", "rain", "graupel", "hail")

    def grow(liquid):
        c0, ex = _g_cell(268.15, 60000, q=4.5e-3, cloud=0.4 * liquid, rain=0.6 * liquid, hail=5e-3)
        before = sum(f32(c0.get(k, 0)) for k in species)
        _, c = O.cell("hail", c0, exner=ex, p=60000, rho=0.8, dt=5)
        grown = float(c["hail"]) - f32(5e-3)
        assert close((float(c["theta"]) - f32(c0["theta"])) * ex, LF / CP * grown, 4)
        assert close(sum(float(c[k]) for k in species), before, 9)
        return grown
    a, b = grow(8e-3), grow(16e-3)
    assert a > 0 and b / a < 1.2


def test_hail_melts_above_zero():  # :55-61
    c0, ex = _g_cell(283.15, 85000, q=6e-3, hail=3e-3)
    cool, c = O.cell("hail", c0, exner=ex, p=85000, rho=1, dt=10)
    assert c["rain"] > 0 and close(float(c["rain"]) + float(c["hail"]), 3e-3, 9)
    assert close(cool * ex, LF / CP * float(c["rain"]), 5)


# ------------------------------------------------------------------ src/core/spectral.test.ts
class _Lehmer:
    def __init__(self):
        self.seed = 12345

    def __call__(self):
        self.seed = (self.seed * 16807) % 2147483647
        return self.seed / 2147483647 - 0.5


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 20, 32, 40, 64, 80])
def test_fft_matches_direct_dft(n):  # :9-20
    r = _Lehmer()
    re = np.array([r() for _ in range(n)]); im = np.array([r() for _ in range(n)])
    f_re, f_im = re.copy(), im.copy()
    L.orc_fft(n, O.dp(f_re), O.dp(f_im), -1)
    j = np.arange(n)
    for k in range(n):
        t = -2 * np.pi * j * k / n
        a = np.sum(re * np.cos(t) - im * np.sin(t)); b = np.sum(re * np.sin(t) + im * np.cos(t))
        assert close(f_re[k], a, 10) and close(f_im[k], b, 10)
    L.orc_fft(n, O.dp(f_re), O.dp(f_im), 1)
    assert np.all(np.abs(f_re / n - re) < 0.5e-12) and np.all(np.abs(f_im / n - im) < 0.5e-12)


@pytest.mark.parametrize("nx,ny", [(1, 1), (4, 1), (5, 3), (8, 6), (40, 32)])
def test_horizontal_dft_inverts(nx, ny):  # :23-33
    r = _Lehmer(); layers = 2
    src = np.array([r() for _ in range(nx * ny * layers)])
    re, im, out = np.empty_like(src), np.empty_like(src), np.empty_like(src)
    L.orc_hdft(nx, ny, layers, O.dp(src), O.dp(re), O.dp(im), O.dp(out))
    m, n, base = nx // 2, min(1, ny - 1), nx * ny
    x, y = np.meshgrid(np.arange(nx), np.arange(ny))
    t = -2 * np.pi * (m * x / nx + n * y / ny)
    vals = src[base:base + nx * ny].reshape(ny, nx)
    assert close(re[base + n * nx + m], np.sum(vals * np.cos(t)), 10)
    assert close(im[base + n * nx + m], np.sum(vals * np.sin(t)), 10)
    assert np.all(np.abs(out - src) < 0.5e-12)


# ------------------------------------------------------------------ src/core/pressure.test.ts
PRESSURE_CASES = [(1, 1, 4, None), (4, 1, 3, None), (4, 4, 4, None), (8, 6, 5, None), (12, 10, 24, None),
                  (40, 32, 24, None), (4, 4, 4, 1000.0), (8, 6, 12, 200.0), (12, 10, 40, 100.0)]


@pytest.mark.parametrize("nx,ny,nz,bottom", PRESSURE_CASES)
@pytest.mark.parametrize("anelastic", [False, True])
def test_pressure_solver_removes_divergence(nx, ny, nz, bottom, anelastic):  # :7-26
    grid = create_grid(GridOptions(nx, ny, nz, nx * 1200.0, ny * 1125.0, 15_000.0, bottom))
    rho = 1.2 * np.exp(-grid.zs / 8400) if anelastic else np.ones(nz)
    r = _Lehmer()
    u = np.array([r() for _ in range(grid.n)], np.float32)
    v = np.array([r() for _ in range(grid.n)], np.float32)
    w = np.array([r() for _ in range(grid.n)], np.float32)
    w[:grid.layer] = 0; w[(nz - 1) * grid.layer:] = 0
    cells = nx * ny * (nz - 1)
    d0, d1, p = np.empty(cells), np.empty(cells), np.empty(cells)
    args, keep = O.grid_args(grid)
    rho = O.f64(rho)
    L.orc_pressure_project(*args, O.dp(rho), O.fp(u), O.fp(v), O.fp(w), 1.0, O.dp(d0), O.dp(d1), O.dp(p))
    assert np.all(np.isfinite(p))
    assert np.max(np.abs(d1)) < np.max(np.abs(d0)) * 1e-6


# ------------------------------------------------------------------ src/core/turbulence.test.ts
def _turb_grid():
    return create_grid(GridOptions(16, 12, 8, 16 * 1200.0, 12 * 1125.0, 7 * 652.0))


def _turbulence(grid, rho, u, v, w, theta, theta_env, cs, dt, q=None, cond=None, exner=None, anisotropic=0,
                vertical_dz=0, implicit=0, dk=0, km_in=None, kh_in=None, a=None, base=None, factor=1.0, steps=0):
    args, keep = O.grid_args(grid)
    km, kh = np.empty(grid.n), np.empty(grid.n)
    rho, theta_env = O.f64(rho), O.f64(theta_env)
    exner = None if exner is None else O.f64(exner)
    base = None if base is None else O.f64(base)
    L.orc_turbulence(*args, O.dp(rho), O.fp(u), O.fp(v), O.fp(w), O.fp(theta), O.dp(theta_env), cs, dt, O.fp(q), O.fp(cond),
                     O.dp(exner), anisotropic, vertical_dz, implicit, dk, O.dp(km_in), O.dp(kh_in), O.dp(km), O.dp(kh),
                     O.fp(a), O.dp(base), factor, steps)
    return km, kh


def _field(grid, fn):
    i = np.arange(grid.n)
    return np.array([fn(k % grid.nx, (k // grid.nx) % grid.ny, k // grid.layer) for k in i], np.float32)


def test_turbulence_mixes_only_where_flow_deforms():  # :11-18
    grid = _turb_grid()
    rho = 1.2 * np.exp(-np.arange(grid.nz) * grid.dz / 8400)
    u = _field(grid, lambda x, y, z: 10 * math.sin(2 * math.pi * y / grid.ny) * (1 if 0 < z < grid.nz - 1 else 0))
    zero = np.zeros(grid.n, np.float32)
    km, _ = _turbulence(grid, rho, u, zero, zero, np.full(grid.n, 300, np.float32), np.full(grid.nz, 300.0), 0.18, 1)
    assert km.max() > 50
    stable = 300 + np.arange(grid.nz) * grid.dz * 0.004
    km, _ = _turbulence(grid, rho, np.full(grid.n, 5, np.float32), zero, zero, _field(grid, lambda x, y, z: stable[z]), stable, 0.18, 1)
    assert km.max() == 0


def test_turbulence_smooths_and_conserves_mass():  # :20-29
    grid = _turb_grid()
    rho = 1.2 * np.exp(-np.arange(grid.nz) * grid.dz / 8400)
    u = _field(grid, lambda x, y, z: 10 * math.sin(2 * math.pi * y / grid.ny) * (1 if 0 < z < grid.nz - 1 else 0))
    zero = np.zeros(grid.n, np.float32)
    km, kh = _turbulence(grid, rho, u, zero, zero, np.full(grid.n, 300, np.float32), np.full(grid.nz, 300.0), 0.18, 1)
    q = _field(grid, lambda x, y, z: 1.0 if (x == 8 and y == 0 and z == 3) else 0.0)
    zz = np.arange(grid.n) // grid.layer
    weight = rho[zz] * np.where((zz == 0) | (zz == grid.nz - 1), 0.5, 1.0)
    before = float(np.sum(q * weight))
    _turbulence(grid, rho, u, zero, zero, zero, np.full(grid.nz, 300.0), 0.18, 1, km_in=km, kh_in=kh, a=q,
                base=np.zeros(grid.nz), factor=3, steps=200)
    assert q.max() < 0.9 and q.min() >= 0
    assert abs(float(np.sum(q.astype(np.float64) * weight)) / before - 1) < 1e-4


def test_turbulence_cap_and_vertical_length():  # :58-68
    tall = create_grid(GridOptions(6, 5, 30, 6 * 2000.0, 5 * 2000.0, 15_000.0, 100.0))
    rho = 1.2 * np.exp(-tall.zs / 8400)
    uu = np.array([0.02 * tall.zs[i // tall.layer] for i in range(tall.n)], np.float32)
    zero = np.zeros(tall.n, np.float32); th = np.full(tall.n, 300, np.float32); neutral = np.full(tall.nz, 300.0)

    def k(vdz, implicit):
        km, _ = _turbulence(tall, rho, uu, zero, zero, th, neutral, 0.18, 3, anisotropic=1, vertical_dz=vdz, implicit=implicit)
        return km[2 * tall.layer]
    cap = 0.05 * min(tall.dzs[1], tall.dzs[2]) ** 2 / 3
    assert close(k(0, 0), cap, 6)
    assert k(0, 1) > 1.5 * cap
    assert k(1, 0) < cap / 5

    def iso(vdz):
        _, kh = _turbulence(tall, rho, uu, zero, zero, th, neutral, 0.18, 3, vertical_dz=vdz)
        return kh[2 * tall.layer]
    assert iso(1) == iso(0)


def test_turbulence_durran_klemp_stability():  # :86-105
    grid = _turb_grid()
    rho = 1.2 * np.exp(-np.arange(grid.nz) * grid.dz / 8400)
    exner = np.full(grid.nz, 0.97)
    theta = _field(grid, lambda x, y, z: 300 + 1.5e-3 * grid.zs[z])
    shear = _field(grid, lambda x, y, z: 0.01 * grid.zs[z])
    q = np.full(grid.n, 0.012, np.float32); cond = np.full(grid.n, 1e-3, np.float32)
    calm = np.zeros(grid.n, np.float32); env = np.full(grid.nz, 300.0)
    mid = 3 + grid.nx * 3 + 4 * grid.layer
    km, _ = _turbulence(grid, rho, shear, calm, calm, theta, env, 0.18, 1, q=q, cond=cond, exner=exner)
    assert km[mid] == 0
    km, _ = _turbulence(grid, rho, shear, calm, calm, theta, env, 0.18, 1, q=q, cond=cond, exner=exner, dk=1)
    assert km[mid] > 1
    l2 = (0.18 * np.cbrt(grid.dx * grid.dy * grid.hz[4])) ** 2
    n2 = (1e-4 - (km[mid] / l2) ** 2) / 3
    assert 2.1e-5 < n2 < 2.5e-5
    loaded = _field(grid, lambda x, y, z: 1e-3 + 1e-6 * grid.zs[z])
    km2, _ = _turbulence(grid, rho, shear, calm, calm, theta, env, 0.18, 1, q=q, cond=loaded, exner=exner, dk=1)
    assert km2[mid] > km[mid]


# ------------------------------------------------------------------ src/core/grid.test.ts, model.test.ts:66-70
def test_grid_uniform_and_stretched():
    g = create_grid(GridOptions(40, 32, 30, 48_000.0, 36_000.0, 18_900.0, None))
    assert g.uniform and close(g.zs[-1], g.height, 9)
    assert np.all(g.dzs == g.dz)
    assert g.hz[0] == g.dz / 2 and g.hz[5] == g.dz and g.hz[-1] == g.dz / 2
    g = create_grid(GridOptions(40, 32, 40, 48_000.0, 36_000.0, 18_900.0, 100.0))
    assert not g.uniform and g.zs[0] == 0 and close(g.zs[-1], g.height, 6) and close(g.dzs[0], 100, 6)
    assert np.all(np.diff(g.dzs) > 0)
    assert close(g.hz.sum(), g.height, 6)
    for k in (0, 3, 17, 39):
        assert close(level_at(g, g.zs[k]), k, 9)
    assert close(level_at(g, (g.zs[4] + g.zs[5]) / 2), 4.5, 9)
    d = create_grid(DEFAULT_GRID)
    assert (d.dx, d.dy) == (1200, 1125) and d.nz == 50 and close(d.dzs[0], 100, 6) and close(d.zs[-1], 18_900, 6)
