"""The reference's electrification and lightning tests on the oracle (CPU).

These pin the oracle's restatement of the charging (src/core/charge.test.ts), the lightning (src/core/lightning.test.ts)
and the electrified model (src/core/electrification.test.ts), which the device's charging, charge transport and
discharge are checked against. The Takahashi table both compile in is checked entry for entry against the reference's
own (tests/golden/takahashi_table.json, written by tests/golden/make_takahashi_fixture.py).
"""
import json
import math
import os
import re

import numpy as np
import pytest

import pyoracle as O
from charge_cases import AIR, DT, GRID, mixed_phase, quiet_electrified, separated_charge, storm, total, with_fields

HERE = os.path.dirname(os.path.abspath(__file__))


def close(a, b, digits):
    """vitest's toBeCloseTo(b, digits): |a - b| < 10^-digits / 2."""
    return abs(a - b) < 10 ** -digits / 2


# ------------------------------------------------------------------ the table
def test_takahashi_table_is_the_references():
    ref = json.load(open(os.path.join(HERE, "golden", "takahashi_table.json")))
    text = open(os.path.join(HERE, "..", "meteolab_gb300", "csrc", "sg_takahashi.h")).read()
    lwc = [float(s) for s in re.search(r"SG_TAKAHASHI_LWC \{([^}]*)\}", text).group(1).split(",")]
    body = text[text.index("SG_TAKAHASHI_TABLE"):]
    rows = [[float(s) for s in r.split(",")] for r in re.findall(r"\{ ([^{}]*) \}", body)]
    assert lwc == ref["lwc"]
    assert rows == ref["table"]
    # the lookup reads the table: at a whole degree and a tabulated cloud water it returns the entry itself
    assert O.takahashi(-10, 0.4) == ref["table"][12][10]
    assert O.takahashi(-3, 2.0) == ref["table"][19][3]
    # none at 0 degC and warmer, at -40 and colder, under 0.01 g/m3; colder than -30 the -30 value tapered
    assert O.takahashi(0, 1) == 0 and O.takahashi(-40, 1) == 0 and O.takahashi(-10, .005) == 0
    assert close(O.takahashi(-35, 1.0), ref["table"][18][30] * (1 - .25), 12)


# ------------------------------------------------------------------ charge.test.ts
def test_critical_rime_accretion_rate():  # charge.test.ts:5-11
    R = O.critical_rar
    assert close(R(-7.35), 1.14, 2) and close(R(-10), 1.19, 2) and close(R(-15), 1.65, 2)
    for t in range(-8, -24, -1):
        assert R(t) > R(t + 1)
    assert close(R(-20), 2.76, 1) and close(R(-23.7), 3.39, 1)
    assert R(-2) == R(-7.35) and R(-30) == R(-23.7)


def test_collision_charge():  # :13-33
    q = O.collision_charge
    for d in (155e-6, 452e-6):
        below, above = q(-15, 3, d * (1 - 1e-9), 3), q(-15, 3, d, 3)
        assert close(above / below, 1, 2)
    assert q(-10, 3, 100e-6, 5) > 0
    assert q(-20, 1, 100e-6, 5) < 0

    def ratio(d, v):
        return q(-20, 1, d, v, True) / q(-20, 1, d, v, False)
    assert close(ratio(100e-6, 2), 5.24e8 * 100e-6 ** 2.54 * 2 ** 2.8 / (4.92e13 * 100e-6 ** 3.76 * 2 ** 2.5), 6)
    assert ratio(50e-6, 2) > 2 and ratio(300e-6, .5) < 1
    assert close(q(-20, 1, 253e-6 * (1 - 1e-9), 3, True) / q(-20, 1, 253e-6, 3, True), 1, 2)
    assert q(-10, 3, 100e-6, 5, True) == q(-10, 3, 100e-6, 5, False)
    assert abs(q(-20, 1.4, 100e-6, 5)) > 1e-16 and abs(q(-20, 1.4, 100e-6, 5)) <= 20e-15
    assert q(1, 3, 100e-6, 5) == 0 and q(-35, 3, 100e-6, 5) == 0 and q(-15, .05, 100e-6, 5) == 0
    assert abs(q(-15, 20, 3e-3, 30)) == 20e-15


def test_charging_needs_cloud_water_crystals_and_rimers():  # :35-73
    C = O.charging_rate
    rho = .7
    args = (rho, 1e-3, 5e-4, 5e-4, 2e-3, 0, .8)
    assert C(-15, *args) != 0
    assert C(-15, rho, 0, 5e-4, 5e-4, 2e-3, 0, .8) == 0
    assert C(-15, rho, 1e-3, 0, 0, 2e-3, 0, .8) == 0
    assert C(-15, rho, 1e-3, 5e-4, 5e-4, 0, 0, .8) == 0
    assert C(5, *args) == 0
    sp = dict(scheme="sp98")
    assert C(-20, rho, 2e-4, 5e-4, 5e-4, 2e-3, 0, .8, **sp) < 0
    assert C(-10, rho, 2e-3, 5e-4, 5e-4, 2e-3, 0, .8, **sp) > 0
    assert C(-20, 1, 1.5e-3, 5e-4, 5e-4, 2e-3, 0, .8, **sp) > 0
    assert C(-20, 1, .5e-3, 5e-4, 5e-4, 2e-3, 0, .8, **sp) < 0
    assert C(-10, 1, .4e-3, 5e-4, 5e-4, 2e-3, 0, .8, scheme="tak") > 0
    assert C(-15, 1, 2e-3, 5e-4, 5e-4, 2e-3, 0, .8, scheme="tak") < 0
    assert C(-35, 1, .4e-3, 5e-4, 5e-4, 2e-3, 0, .8, **sp) == 0
    assert C(-35, 1, .4e-3, 5e-4, 5e-4, 2e-3, 0, .8, scheme="tak") != 0
    assert C(-10, rho, 2e-3, 5e-4, 5e-4, 2e-3, 0, .8, True) == 0
    per_minute = abs(C(-20, rho, 3e-4, 1.4e-3, 1e-3, 1.4e-3, 0, .8)) * 60
    assert 1e-11 < per_minute < 1e-8
    assert 50e-6 < O.crystal_diameter(1e-3, rho, -20) < 300e-6 + 1e-12
    assert 100e3 < O.crystal_number(-6, 3e-4, rho) <= 150e3
    assert O.crystal_number(-6, 0, rho) < 100 and O.crystal_number(-35, 1e-6, rho) > 1e4


def test_charge_follows_the_mass_between_carriers():  # :75-102
    T = O.transfer_charge
    c = T([0, 0, 2e-9, 0], [0, 0, 1e-3, 0], [0, 5e-4, 5e-4, 0])
    assert close(c[2], 1e-9, 20) and close(c[1], 1e-9, 20)
    assert list(T([0, -3e-9, 0, 0], [0, 1e-3, 0, 0], [0, 0, 1e-3, 0])) == [0, 0, -3e-9, 0]
    c = T([4e-9, 0, 0, 0], [1e-3, 0, 0, 0], [5e-4, 0, 0, 0])
    assert close(c[0], 2e-9, 20) and close(c[3], 2e-9, 20)
    c = T([0, 8e-9, 0, 0], [0, 2e-3, 0, 0], [0, 1e-3, 2.5e-4, 0])
    assert close(c[1], 4e-9, 20) and close(c[2], 1e-9, 20) and close(c[3], 3e-9, 20)
    c = T([0, 0, 0, 6e-9], [0, 1e-3, 0, 1e-3], [0, 1.5e-3, 0, 5e-4])
    assert close(c[1], 3e-9, 20) and close(c[3], 3e-9, 20)
    assert list(T([1e-9, 0, 0, 0], [1e-3, 0, 0, 0], [2e-3, 0, 0, 0])) == [1e-9, 0, 0, 0]
    c = T([0, 5e-12, 0, 2e-12], [0, 0, 0, 0], [0, 0, 0, 0])
    assert c[1] == 0 and close(c[3], 7e-12, 25)
    c0 = [3e-9, -5e-9, 1e-9, -2e-10]
    c = T(c0, [1e-3, 2e-3, 5e-4, 3e-4], [2e-4, 2.6e-3, 0, 1e-4])
    assert close(sum(c), sum(c0), 22)


def test_inductive_charging():  # :105-118
    I = O.inductive_rate
    rho = .7
    per_minute = I(-10, rho, 1e-3, 2.9e-3, 0, 5e4, 0) * 60
    assert .2e-9 < per_minute < 5e-9
    assert close(I(-10, rho, 1e-3, 2.9e-3, 0, -5e4, 0), -per_minute / 60, 15)
    relax = I(-10, rho, 1e-3, 2.9e-3, 0, 0, 1e-9)
    assert relax < 0 and 30 < 1e-9 / -relax < 1000
    assert I(-10, rho, 0, 2.9e-3, 0, 5e4, 0) == 0 and I(-10, rho, 1e-3, 0, 0, 5e4, 0) == 0
    assert I(-10, rho, 1e-3, 2.9e-3, 0, 5e4, 0, True) == 0 and I(5, rho, 1e-3, 2.9e-3, 0, 5e4, 0) == 0


# ------------------------------------------------------------------ lightning.test.ts
def test_tripole_discharges_inside_the_cloud():  # lightning.test.ts:33-55
    carriers = storm([[10000, 2], [6500, -3.5], [3500, 1]])
    before = [c.copy() for c in carriers]
    start = total(carriers)
    L = O.OracleLightning(GRID, AIR, 7)
    L.solve(carriers)
    assert L.strongest()[1] > 1
    flashes = L.discharge(carriers, 0)
    assert flashes
    first = flashes[0]
    height = GRID.zs[first["start"] // GRID.layer]
    assert first["kind"] == "IC"
    assert 6500 < height < 10000
    assert (first["polarity"] > 0).any() and (first["polarity"] < 0).any()
    assert 3 < first["charge"] < 100
    assert abs(total(carriers) - start) < 1e-6 * first["charge"]
    for k in range(4):
        assert (carriers[k].astype(np.float64) * before[k] >= 0).all()
    L.solve(carriers)
    assert L.strongest()[1] < 1


def test_negative_cg_without_the_lower_positive_charge():  # :57-72
    carriers = storm([[9000, 3], [6500, -3]])
    start = total(carriers)
    L = O.OracleLightning(GRID, AIR, 7)
    flashes = L.discharge(carriers, 0)
    first = flashes[0]
    assert first["kind"] == "CG" and first["charge"] < 0
    assert 0 <= first["ground"] < GRID.layer
    assert first["parent"][0] == -1 and len(first["polarity"]) == len(first["nodes"])
    for c in range(1, len(first["nodes"])):
        assert 0 <= first["parent"][c] < c
    lowered = sum(f["charge"] for f in flashes if f["kind"] == "CG")
    from_ground = L.fields()[2]["fromGround"]
    assert close(from_ground, -lowered, 6)
    assert abs(total(carriers) - start - from_ground) < 1e-6 * abs(first["charge"])


def test_below_the_threshold_nothing_happens():  # :88-92
    carriers = storm([[9000, .5], [6500, -.5]])
    before = [c.copy() for c in carriers]
    assert O.OracleLightning(GRID, AIR, 7).discharge(carriers, 0) == []
    for a, b in zip(carriers, before):
        assert np.array_equal(a, b)


def test_flash_limit():  # :94-101
    assert [O.flash_limit(d) for d in (3, 6, 1.5, .75, .1)] == [10, 20, 5, 3, 1]
    strong = lambda: storm([[10000, 8], [6500, -14], [3500, 4]])  # noqa: E731
    assert len(O.OracleLightning(GRID, AIR, 7).discharge(strong(), 0, 50)) > 2
    assert len(O.OracleLightning(GRID, AIR, 7).discharge(strong(), 0, 2)) == 2


def centre(z):
    return GRID.nx // 2 + GRID.ny // 2 * GRID.nx + z * GRID.layer


def level(m):
    return int(np.argmax(np.asarray(GRID.zs) >= m))


def net(carriers, i):
    return sum(float(c[i]) for c in carriers)


def test_conduction_relaxes_clear_air_charge():  # :110-122
    carriers = storm([[10000, 1]])
    start = total(carriers)
    L = O.OracleLightning(GRID, AIR, 7)
    z = level(10000)
    before = net(carriers, centre(z))
    L.solve(carriers)
    lost = L.conduct(carriers[3], 10)
    relaxed = 1 - net(carriers, centre(z)) / before
    assert .05 < relaxed < .15
    assert lost == L.fields()[2]["conducted"]
    assert abs(total(carriers) - start + lost) < 1e-9 * abs(start)


def test_screening_layer_at_the_cloud_edge():  # :124-137
    nx, ny, nz = GRID.nx, GRID.ny, GRID.nz
    carriers = storm([[10000, 1]])
    L = O.OracleLightning(GRID, AIR, 7)
    cloudy = np.zeros(GRID.n, np.float32)
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                if math.hypot((x - nx // 2) * GRID.dx, (y - ny // 2) * GRID.dy) < 4000 and abs(GRID.zs[z] - 10000) < 1500:
                    cloudy[x + y * nx + z * GRID.layer] = 1e-3
    z = level(10000)
    before = net(carriers, centre(z))
    L.cloud([cloudy])
    for _ in range(60):
        L.solve(carriers)
        L.conduct(carriers[3], 10)
    assert net(carriers, centre(z)) / before > .3
    top, side = level(11500 + 200), round(4000 / GRID.dx) + 1
    assert net(carriers, centre(top)) < 0
    assert net(carriers, nx // 2 + side + ny // 2 * nx + z * GRID.layer) < 0


def test_corona_under_a_negative_charge():  # :139-157
    carriers = storm([[5000, -4]])
    start = total(carriers)
    L = O.OracleLightning(GRID, AIR, 7)
    L.solve(carriers)
    field = -L.fields()[0][centre(1)] / GRID.dzs[0]
    assert field > 5e3
    lost = L.conduct(carriers[3], 10)
    assert net(carriers, centre(1)) > 0
    assert abs(total(carriers) - start + lost) < 1e-9 * abs(start)
    weak = storm([[5000, -.01]])
    quiet = O.OracleLightning(GRID, AIR, 7)
    quiet.solve(weak)
    assert abs(quiet.fields()[0][centre(1)] / GRID.dzs[0]) < 5e3
    sea = storm([[5000, -4]])
    wet = O.OracleLightning(GRID, AIR, 7)
    wet.set_corona(False)
    wet.solve(sea)
    wet.conduct(sea[3], 10)
    assert net(sea, centre(1)) < .1 * net(carriers, centre(1))


# ------------------------------------------------------------------ electrification.test.ts on the oracle's model
def model_with(spec, fields, fp64=False):
    return O.OracleModel(with_fields(spec, fields), fp64=fp64)


def test_collisions_separate_charge_and_the_domain_stays_neutral():  # electrification.test.ts:20-33
    spec = quiet_electrified()
    m = model_with(spec, mixed_phase(spec))
    m.step(DT, 10)
    sep = separated_charge(m.get, spec)
    assert sep > 0
    graupel, ice = float(np.sum(m.get("chargeGraupel"))), float(np.sum(m.get("chargeIce")))
    assert abs(graupel) > 0 and np.sign(graupel) == -np.sign(ice)
    st = m.charge_state()
    assert abs(st["totalCharge"] + st["chargeGround"]) < 1e-5 * sep


def test_a_charged_block_falls_with_its_carriers():  # :35-47
    spec = quiet_electrified()
    f = mixed_phase(spec, 8000, 9500)
    f["cloud"][:] = 0
    g = spec.grid
    cg = np.zeros(g.n)
    for i in np.nonzero(f["graupel"] > 0)[0]:
        cg[i] = np.float32(1e-9 / spec.env.rho[i // g.layer])
    f["chargeGraupel"] = cg
    m = model_with(spec, f)
    start = m.charge_state()["totalCharge"]
    zs = np.repeat(np.asarray(g.zs), g.layer)

    def height(c):
        return float(np.sum(c * zs) / np.sum(c))
    h0 = height(m.get("chargeGraupel"))
    m.step(DT, 20)
    st = m.charge_state()
    assert abs(st["totalCharge"] + st["chargeGround"] - start) / start < 1e-4
    assert h0 - height(m.get("chargeGraupel")) > 150


def test_a_strongly_charged_cloud_flashes_and_conserves_charge():  # :49-64
    spec = quiet_electrified()
    g, rho = spec.grid, spec.env.rho
    f = {k: v.copy() for k, v in spec.fields.items()}
    nx, ny = g.nx, g.ny
    zs = np.asarray(g.zs)[:, None, None]
    y = np.arange(ny)[None, :, None]
    x = np.arange(nx)[None, None, :]
    r2 = ((x - nx // 2) * g.dx) ** 2 + ((y - ny // 2) * g.dy) ** 2
    air = np.asarray(rho)[:, None, None]
    f["chargeIce"] = (3e-9 * np.exp(-r2 / 2500 ** 2 - ((zs - 9000) / 700) ** 2) / air).astype(np.float32).ravel()
    f["chargeGraupel"] = (-3e-9 * np.exp(-r2 / 2500 ** 2 - ((zs - 6500) / 700) ** 2) / air).astype(np.float32).ravel()
    m = model_with(spec, f)
    start = m.charge_state()["totalCharge"]
    m.step(DT, 1)
    flashes = m.last_flashes()
    st = m.charge_state()
    assert len(flashes) > 0
    assert st["flashesIC"] + st["flashesCG"] == len(flashes)
    assert all(fl["time"] == DT for fl in flashes)
    assert abs(st["totalCharge"] + st["chargeGround"] - start) < 1e-3


def test_switched_off_no_charge_appears():  # :66-71
    for lightning in (False, True):
        spec = quiet_electrified(lightning=lightning)
        if lightning:  # without the ice microphysics nothing charges either
            spec.switches.ice = 0
        m = model_with(spec, mixed_phase(spec))
        m.step(DT, 5)
        assert not np.any(m.get("chargeGraupel")) and not np.any(m.get("chargeIce"))
