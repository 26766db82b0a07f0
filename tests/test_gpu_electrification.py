"""Electrification and lightning on the device, against the oracle (GPU).

* The discharge alone (AtmosphereModel.discharge through sg_run_discharge) on the reference's charge regions: the
  same flashes as the oracle's Lightning (kind, initiation node, channel node for node, charge), the carriers after
  them, the conduction. The channel grows by the same random picks over the same weights; the potential it grows on
  is the device's FP64 solve (direct DFTs) against the oracle's (FFTs), equal to ~1e-12 of its range, so a pick can
  differ only where a random number falls within that of a weight boundary.
* The electrified step: ten steps of the reference's mixed-phase cloud block (electrification.test.ts:20-33) against
  the oracle model: the charge carriers to 2e-4 relative L2 (the charging rates are FP32 on the device and the oracle's
  FP64, and their thresholds -- wet growth, the Takahashi table's rows -- fall on a node's FP32 state), the domain
  neutral to 1e-5 of the separated charge as in the reference.
* The charge falls with its carriers and is conserved (:35-47); a strongly charged cloud flashes in its first step,
  each flash timed at the step's end, and the charge with what went to the ground is conserved (:49-64).
* Electrification changes no other field: an electrified run's 13 carried fields are the bits of the same run
  without it.
"""
import numpy as np
import pytest

import pyoracle as O
from charge_cases import AIR, DT, GRID, mixed_phase, quiet_electrified, separated_charge, storm, total, total_charge, tripole_with_cloud, with_fields
from parity import rel_l2
from meteolab_gb300.scenarios import CARRIED, CHARGES, baseline_run

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import Context
    c = Context()
    yield c
    c.close()


def oracle_discharge(spec, time, dt):
    """The oracle's AtmosphereModel.discharge on the spec's fields: cloud([cloud, ice, snow]), the flashes, conduct."""
    carriers = [np.array(spec.fields[k], np.float32) for k in CHARGES]  # copies: the oracle changes them in place
    L = O.OracleLightning(GRID, spec.env.rho, spec.switches.lightning_seed)
    L.cloud([np.ascontiguousarray(spec.fields[k], np.float32) for k in ("cloud", "ice", "snow")])
    flashes = L.discharge(carriers, time, O.flash_limit(dt))
    lost = L.conduct(carriers[3], dt)
    return flashes, carriers, lost


def test_field_and_breakdown_search_match_the_oracle(ctx):
    """The discharge's first search: the charge density, its FP64 potential and the strongest field's node."""
    spec = tripole_with_cloud([[10000, 2], [6500, -3.5], [3500, 1]])
    r = ctx.create(spec)
    phi, rho, best, ratio, _ = r.lightning_probe()
    L = O.OracleLightning(GRID, spec.env.rho, 43)
    carriers = [np.array(spec.fields[k], np.float32) for k in CHARGES]
    L.solve(carriers)
    ophi, orho, _ = L.fields()
    obest, oratio = L.strongest()
    print(f"\nprobe: device best {best} ratio {ratio:.9f}, oracle best {obest} ratio {oratio:.9f}; "
          f"rho err {np.max(np.abs(rho - orho)) / np.max(np.abs(orho)):.2e}, phi err {np.max(np.abs(phi - ophi)) / np.max(np.abs(ophi)):.2e}")
    assert np.max(np.abs(rho - orho)) <= 1e-15 * np.max(np.abs(orho))
    assert np.max(np.abs(phi - ophi)) <= 1e-10 * np.max(np.abs(ophi))
    assert best == obest and abs(ratio - oratio) <= 1e-9 * oratio
    r.retire()


@pytest.mark.parametrize("regions,everywhere,seed,time,kind", [([[10000, 2], [6500, -3.5], [3500, 1]], False, 43, DT, "IC"),
                                                                ([[9000, 3], [6500, -3]], False, 43, DT, "IC"),
                                                                ([[9000, 3], [6500, -3]], True, 7, 0.0, "CG")])
def test_discharge_matches_the_oracle_lightning(ctx, regions, everywhere, seed, time, kind):
    """kind: the first flash's. The dipole discharges inside its cloud when the air below is clear; with cloud
    everywhere (clear air known by its charge alone) and the reference test's seed and time its negative charge goes
    to the ground (lightning.test.ts:57-72)."""
    import dataclasses
    spec = tripole_with_cloud(regions, everywhere)
    spec.switches = dataclasses.replace(spec.switches, lightning_seed=seed)
    ref_flashes, ref_carriers, ref_lost = oracle_discharge(spec, time, DT)
    r = ctx.create(spec)
    start = total_charge(lambda k: spec.fields[k], spec)
    r.discharge(time, DT)
    got = r.flashes()
    print(f"\n{kind}: device {[(f['kind'], f['start'], len(f['nodes']), round(f['charge'], 4)) for f in got]}")
    print(f"{kind}: oracle {[(f['kind'], f['start'], len(f['nodes']), round(f['charge'], 4)) for f in ref_flashes]}")
    assert len(got) == len(ref_flashes) and len(got) > 0
    assert got[0]["kind"] == kind
    for a, b in zip(got, ref_flashes):
        assert a["kind"] == b["kind"] and a["start"] == b["start"] and a["ground"] == b["ground"]
        assert np.array_equal(a["nodes"], b["nodes"]) and np.array_equal(a["parent"], b["parent"])
        assert np.array_equal(a["polarity"], b["polarity"])
        assert abs(a["charge"] - b["charge"]) <= 1e-6 * abs(b["charge"])
        assert a["time"] == time
    fields = r.read(list(CHARGES))
    scale = max(float(np.max(np.abs(c))) for c in ref_carriers)
    for k, ref in zip(CHARGES, ref_carriers):
        assert float(np.max(np.abs(fields[k].astype(np.float64) - ref))) <= 1e-5 * scale, k
    # conservation: what the flashes took from the ground and the conduction gave it
    st = r.charge()
    end = total_charge(lambda k: fields[k], spec)
    assert abs(end + st["ground"] - start) < 1e-6 * max(abs(f["charge"]) for f in got)
    assert abs(st["conduction"] - ref_lost) <= 1e-6 * abs(ref_lost) + 1e-15
    assert st["flashes_ic"] + st["flashes_cg"] == len(got)
    r.retire()


def test_below_the_threshold_no_flash(ctx):
    spec = tripole_with_cloud([[9000, .5], [6500, -.5]])
    r = ctx.create(spec)
    r.discharge(DT, DT)
    assert r.flashes() == []
    r.retire()


def test_electrified_step_matches_the_oracle(ctx):
    spec = quiet_electrified()
    fields = mixed_phase(spec)
    s2 = with_fields(spec, fields)
    o = O.OracleModel(s2)
    r = ctx.create(s2)
    o.step(DT, 10)
    r.step(10)
    got = r.read(list(CARRIED) + list(CHARGES))
    errs = {k: rel_l2(got[k], o.get(k)) for k in CHARGES}
    norms = {k: float(np.linalg.norm(o.get(k))) for k in CHARGES}
    print("\nchargeparity: " + ", ".join(f"{k} {v:.2e} (norm {norms[k]:.2e})" for k, v in errs.items()))
    for k, e in errs.items():
        # the charge on rain is moved there by the charge transfer in proportion to rain's mass gain in the step,
        # increments of 1e-10..1e-8 kg/kg on ~1e-4 that FP32 microphysics resolves to an ulp of the rain mass
        assert e < (2e-3 if k == "chargeRain" else 2e-4), (k, e)
    sep = separated_charge(lambda k: got[k], spec)
    assert sep > 0
    graupel, ice = float(np.sum(got["chargeGraupel"])), float(np.sum(got["chargeIce"]))
    assert abs(graupel) > 0 and np.sign(graupel) == -np.sign(ice)
    st = r.charge()
    assert abs(total_charge(lambda k: got[k], spec) + st["ground"]) < 1e-5 * sep
    ost = o.charge_state()
    assert abs(st["separated"] - ost["separated"]) <= 1e-3 * ost["separated"]
    r.retire()


def test_charged_block_falls_with_its_carriers(ctx):
    spec = quiet_electrified()
    f = mixed_phase(spec, 8000, 9500)
    f["cloud"][:] = 0
    layer = GRID.layer
    cg = np.zeros(GRID.n, np.float32)
    for i in np.nonzero(f["graupel"] > 0)[0]:
        cg[i] = np.float32(1e-9 / spec.env.rho[i // layer])
    f["chargeGraupel"] = cg
    s2 = with_fields(spec, f)
    r = ctx.create(s2)
    start = total_charge(lambda k: s2.fields[k] if k in s2.fields else np.zeros(GRID.n), s2)
    zs = np.repeat(np.asarray(GRID.zs), layer)

    def height(c):
        c = c.astype(np.float64)
        return float(np.sum(c * zs) / np.sum(c))
    h0 = height(cg)
    r.step(20)
    got = r.read(list(CHARGES))
    st = r.charge()
    assert abs(total_charge(lambda k: got[k], s2) + st["ground"] - start) / start < 1e-4
    assert h0 - height(got["chargeGraupel"]) > 150
    r.retire()


def test_strongly_charged_cloud_flashes_in_its_step(ctx):
    spec = quiet_electrified()
    g, rho = GRID, spec.env.rho
    f = {k: v.copy() for k, v in spec.fields.items()}
    zs = np.asarray(g.zs)[:, None, None]
    y = np.arange(g.ny)[None, :, None]
    x = np.arange(g.nx)[None, None, :]
    r2 = ((x - g.nx // 2) * g.dx) ** 2 + ((y - g.ny // 2) * g.dy) ** 2
    air = np.asarray(rho)[:, None, None]
    f["chargeIce"] = (3e-9 * np.exp(-r2 / 2500 ** 2 - ((zs - 9000) / 700) ** 2) / air).astype(np.float32).ravel()
    f["chargeGraupel"] = (-3e-9 * np.exp(-r2 / 2500 ** 2 - ((zs - 6500) / 700) ** 2) / air).astype(np.float32).ravel()
    s2 = with_fields(spec, f)
    r = ctx.create(s2)
    o = O.OracleModel(s2)
    start = total_charge(lambda k: f.get(k, np.zeros(g.n)), s2)
    r.step(1)
    o.step(DT, 1)
    flashes, ref = r.flashes(channels=False), o.last_flashes()
    print(f"\ndevice {[(a['kind'], round(a['charge'], 3)) for a in flashes]}\noracle {[(b['kind'], round(b['charge'], 3)) for b in ref]}")
    st = r.charge()
    assert len(flashes) > 0
    assert st["flashes_ic"] + st["flashes_cg"] == len(flashes)
    assert all(a["time"] == DT for a in flashes)
    got = r.read(list(CHARGES))
    assert abs(total_charge(lambda k: got[k], s2) + st["ground"] - start) < 1e-3
    # the step before the discharge moved the charges by FP32 rounding only: the same flashes as the oracle's
    assert [a["kind"] for a in flashes] == [b["kind"] for b in ref]
    for a, b in zip(flashes, ref):
        assert abs(a["charge"] - b["charge"]) <= 1e-3 * abs(b["charge"])
    r.retire()


def test_electrification_changes_no_other_field(ctx):
    """A growing storm run with and without electrification: the 13 carried fields are the same bits."""
    base = baseline_run(GRID, seed=5, bubble=3.0)
    on = with_fields(base, base.fields)
    import dataclasses
    on.switches = dataclasses.replace(base.switches, lightning=1)
    a, b = ctx.create(base), ctx.create(on)
    a.step(40)
    b.step(40)
    fa, fb = a.read(), b.read()
    for k in CARRIED:
        assert np.array_equal(fa[k], fb[k]), k
    assert b.charge()["electrified"] == 1 and a.charge()["electrified"] == 0
    a.retire()
    b.retire()


def test_electrified_state_saves_and_loads(ctx):
    """A .meteolab file of an electrified run (state.ts:34-83): the four charge fields in STATE_FIELDS order, the ground
    charge, flash counts and charge budget in the header; a run loaded from it has them all, saves the same bytes, and
    two loaded runs go on flashing alike."""
    import state_format as SF
    spec = quiet_electrified()
    g, rho = GRID, spec.env.rho
    f = {k: v.copy() for k, v in spec.fields.items()}
    zs = np.asarray(g.zs)[:, None, None]
    y = np.arange(g.ny)[None, :, None]
    x = np.arange(g.nx)[None, None, :]
    r2 = ((x - g.nx // 2) * g.dx) ** 2 + ((y - g.ny // 2) * g.dy) ** 2
    air = np.asarray(rho)[:, None, None]
    f["chargeIce"] = (4e-9 * np.exp(-r2 / 2500 ** 2 - ((zs - 9000) / 700) ** 2) / air).astype(np.float32).ravel()
    f["chargeGraupel"] = (-4e-9 * np.exp(-r2 / 2500 ** 2 - ((zs - 6500) / 700) ** 2) / air).astype(np.float32).ravel()
    s2 = with_fields(spec, f)
    r = ctx.create(s2)
    r.step(2)
    cfg = {"seed": 42, "lightning": True}
    img = r.save_state(cfg, persisted=0.0)
    header, fields, _ = SF.read_state(img)
    got = r.read(list(CHARGES))
    for k in CHARGES:
        assert np.array_equal(fields[k], got[k]), k
    st = r.charge()
    assert st["flashes_ic"] + st["flashes_cg"] > 0
    assert header["chargeGround"] == st["ground"]
    assert header["flashCount"] == {"ic": st["flashes_ic"], "cg": st["flashes_cg"]}
    assert header["charge"]["separated"] == st["separated"] and header["charge"]["conduction"] == st["conduction"]
    a, b = ctx.create(s2), ctx.create(s2)
    a.load_state(img)
    b.load_state(img)
    ga = a.read(list(CHARGES))
    for k in CHARGES:
        assert np.array_equal(ga[k], got[k]), k
    sa = a.charge()
    for k in ("ground", "separated", "ic", "cg_negative", "cg_positive", "precipitation", "conduction", "flashes_ic", "flashes_cg"):
        assert sa[k] == st[k], k
    assert a.save_state(cfg, persisted=0.0) == img
    a.step(2)
    b.step(2)
    fa, fb = a.read(list(CARRIED) + list(CHARGES)), b.read(list(CARRIED) + list(CHARGES))
    for k in fa:
        assert np.array_equal(fa[k], fb[k]), k
    assert [(q["kind"], q["start"], q["charge"]) for q in a.flashes(False)] == [(q["kind"], q["start"], q["charge"]) for q in b.flashes(False)]
    for m in (r, a, b):
        m.retire()
