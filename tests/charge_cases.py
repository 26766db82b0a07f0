"""Shared cases of the electrification tests (tests/test_oracle_charge.py on the oracle, tests/test_gpu_electrification.py
on the device): the reference's charge regions (src/core/lightning.test.ts:14-29), its mixed-phase cloud block
(src/core/electrification.test.ts:7-17) and its QUIET configuration (src/core/fixtures.ts:22-25).
"""
import numpy as np

import pyoracle as O
from meteolab_gb300.environment import Environment, SliderConfig
from meteolab_gb300.grid import DEFAULT_GRID, create_grid
from meteolab_gb300.scenarios import RunSpec, Switches, initial_fields

DT = 3.0
# stable, unsaturated, sunless, no bubble
QUIET = dict(lapseLow=6, lapseMid=6, lapseUpper=6, rhSurface=50, rhLow=40, rhMid=30, rhUpper=20)
GRID = create_grid(DEFAULT_GRID)
AIR = Environment(SliderConfig(**QUIET), GRID).rho


def storm(regions, grid=GRID, air=AIR):
    """Gaussian charge regions over the domain centre, [height m, peak nC/m3], 2.5 km wide and 0.7 km deep: positive
    on the ice carrier, negative on the graupel (lightning.test.ts:14-22), as FP32 carriers in C/kg."""
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    zs = np.asarray(grid.zs)[:, None, None]
    y = np.arange(ny)[None, :, None]
    x = np.arange(nx)[None, None, :]
    r2 = ((x - nx // 2) * grid.dx) ** 2 + ((y - ny // 2) * grid.dy) ** 2
    air3 = np.asarray(air)[:, None, None]
    acc = [np.zeros((nz, ny, nx), np.float32) for _ in range(4)]
    for h, peak in regions:
        k = 0 if peak > 0 else 1
        term = peak * 1e-9 * np.exp(-r2 / 2500 ** 2 - ((zs - h) / 700) ** 2) / air3
        acc[k] = (acc[k].astype(np.float64) + term).astype(np.float32)  # Float32Array +=
    return [np.ascontiguousarray(a.ravel()) for a in acc]


def total(carriers, grid=GRID, air=AIR):
    """Charge in the domain, C (lightning.test.ts:25-29)."""
    s = 0.0
    layer = grid.nx * grid.ny
    for z in range(grid.nz):
        w = air[z] * grid.dx * grid.dy * grid.hz[z]
        for c in carriers:
            s += float(np.sum(c[z * layer:(z + 1) * layer].astype(np.float64))) * w
    return s


def quiet_electrified(lightning=True):
    """A QUIET run on the standard grid (no bubble, no noise) with electrification switched on or off."""
    env = Environment(SliderConfig(**QUIET), GRID)
    sw = Switches(lightning=1 if lightning else 0)
    return RunSpec(GRID, env, sw, initial_fields(GRID, env, 1, bubble=0.0, noise=0.0), 1, "quiet")


def mixed_phase(spec, z0=5500, z1=7500):
    """The fields of `spec` with a block of mixed-phase cloud at the levels between z0 and z1, saturated over water
    (electrification.test.ts:7-17)."""
    g, env = spec.grid, spec.env
    f = {k: v.copy() for k, v in spec.fields.items()}
    nx, ny = g.nx, g.ny
    for z in range(g.nz):
        if not (z0 <= g.zs[z] <= z1):
            continue
        for y in range(ny // 2 - 3, ny // 2 + 3):
            for x in range(nx // 2 - 3, nx // 2 + 3):
                i = x + y * nx + z * g.layer
                f["cloud"][i], f["ice"][i], f["snow"][i], f["graupel"][i] = 1e-3, 5e-4, 5e-4, 2e-3
                t = float(f["theta"][i]) * env.exner[z] - 273.15
                f["q"][i] = max(float(f["q"][i]), O.lib().orc_qsat(t, env.p[z]))
    return f


def with_fields(spec, fields):
    return RunSpec(spec.grid, spec.env, spec.switches, fields, spec.seed, spec.label)


def total_charge(get, spec):
    """totalCharge (src/core/model.ts:1555-1560) of a model whose fields `get(name)` returns."""
    g, rho = spec.grid, spec.env.rho
    a, b, c, d = (np.asarray(get(k), np.float64) for k in ("chargeIce", "chargeGraupel", "chargeRain", "chargeAir"))
    s = 0.0
    for z in range(g.nz):
        sl = slice(z * g.layer, (z + 1) * g.layer)
        s += float(np.sum(a[sl] + b[sl] + c[sl] + d[sl])) * rho[z] * g.dx * g.dy * g.hz[z]
    return s


def separated_charge(get, spec):
    """|charge| of the ice, graupel and rain carriers over the nodes' air mass (electrification.test.ts:24-26)."""
    g = spec.grid
    s = 0.0
    a, b, c = (np.asarray(get(k), np.float64) for k in ("chargeIce", "chargeGraupel", "chargeRain"))
    for z in range(g.nz):
        sl = slice(z * g.layer, (z + 1) * g.layer)
        s += float(np.sum(np.abs(a[sl]) + np.abs(b[sl]) + np.abs(c[sl]))) * spec.env.rho[z] * g.dx * g.dy * g.hz[z]
    return s


def tripole_with_cloud(regions, everywhere=False):
    """A QUIET electrified run's fields carrying `regions` of charge, with cloud water where the charge is (so the
    channel knows the cloud by its mixing ratios as the model's lightning does, src/core/model.ts:1541), or
    everywhere (then the channel knows clear air by its charge alone, as the reference's Lightning without cloud())."""
    spec = quiet_electrified()
    f = {k: v.copy() for k, v in spec.fields.items()}
    carriers = storm(regions)
    rho = np.repeat(np.asarray(spec.env.rho), GRID.layer)
    dens = np.abs(sum(c.astype(np.float64) for c in carriers)) * rho
    f["cloud"] = np.full(GRID.n, 1e-3) if everywhere else np.where(dens > 2e-11, 1e-3, 0.0)
    for name, c in zip(("chargeIce", "chargeGraupel", "chargeRain", "chargeAir"), carriers):
        f[name] = c
    return with_fields(spec, f)
