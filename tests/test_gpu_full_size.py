"""The device step at the benchmark's full sizes (GPU). Per field against the FP64 oracle: one step on the large and the
stress grid, and the two switches no other parity case exercises, the wind limits (clipWind) and a moving frame.
Through size-independent properties: the large 80x64x50
domain and the 320x256x80 stress grid (its layer spectrum too wide for shared memory: the row-transform path of the
spectral solves), each grown from a warm bubble for 100 steps (the scope of the large and stress configurations):
every field finite, no wind clipped, the post-projection divergence before its FP32 rounding at rounding level (the
projection's own operators in FP64 on the velocities and the pressure the device returns), water conserved with the
rain gauge to the reference's 1e-4 (src/core/invariants.test.ts:84-94), and the run the same alone and batched."""
import numpy as np
import pytest

import pyoracle as O
from parity import FLOOR, WATER, developed_state, dual_divergence, field_errors, pressure_gradient, rel_l2, threads, water_total
from meteolab_gb300.grid import DEFAULT_GRID, LARGE_GRID, STRESS_GRID, create_grid
from meteolab_gb300.scenarios import CARRIED, baseline_run

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import Context
    c = Context()
    yield c
    c.close()


@pytest.mark.parametrize("opts,label", [(LARGE_GRID, "large 80x64x50"), (STRESS_GRID, "stress 320x256x80")])
def test_a_full_size_run_keeps_the_invariants(ctx, opts, label):
    spec = baseline_run(create_grid(opts), seed=5, bubble=3.0)
    g = spec.grid
    r = ctx.create(spec)
    before = water_total(r.read(WATER), np.zeros(g.layer), spec)
    r.step(99)
    # the 100th step part by part: the velocities before the final projection, then the projection
    for part in (1, 2, 3, 4):
        r.debug_part(part)
    pre = r.read(("u", "v", "w"))
    r.debug_part(5)
    f = r.read()
    for k in CARRIED:
        assert np.isfinite(f[k]).all(), (label, k)
    st = r.status()
    assert st["clipped"] == 0 and not st["failed"]
    # before rounding: v = u - dt G p from the FP32 velocities and the device's pressure, FP64 (the solve's accuracy);
    # after rounding: the stored FP32 velocities (their rounding bounds it, more so on the finer stress grid)
    dt = spec.switches.dt
    gx, gy, gz = pressure_gradient(r.pressure(), g)
    pu, pv, pw = (pre[k].astype(np.float64) for k in ("u", "v", "w"))
    removed = np.max(np.abs(dual_divergence(pu, pv, pw, g, spec.env.rho)))
    exact = np.max(np.abs(dual_divergence(pu - dt * gx, pv - dt * gy, pw - dt * gz, g, spec.env.rho)))
    left = np.max(np.abs(dual_divergence(f["u"].astype(np.float64), f["v"].astype(np.float64), f["w"].astype(np.float64), g, spec.env.rho)))
    print(f"\n{label}: max |D rho u| before the projection {removed:.3e}; after, before rounding {exact / removed:.2e}, "
          f"after rounding {left / removed:.2e}")
    assert exact <= 1e-8 * removed
    assert left <= 1e-4 * removed
    assert float(np.max(np.abs(f["w"]))) > 1.0          # a growing thermal, not a resting state
    after = water_total(f, r.columns()["precipitation"], spec)
    assert abs(after / before - 1) < 1e-4, (label, after / before - 1)
    r.retire()


def test_the_stress_grid_is_the_same_alone_and_in_a_batch(ctx):
    """The stress run (the row-transform path) and a large run (the 2-D layer transforms) each give the bits they get
    alone when batched together: the spectral path is chosen run by run, not by the batch's widest grid."""
    big = baseline_run(create_grid(STRESS_GRID), seed=6, bubble=2.0)
    small = baseline_run(create_grid(LARGE_GRID), seed=7)
    a, b = ctx.create(big), ctx.create(small)
    a.step(5)
    b.step(5)
    x, y = ctx.create(big), ctx.create(small)
    ctx.batch_step([x, y], 5)
    fa, fb, fx, fy = a.read(), b.read(), x.read(), y.read()
    for k in CARRIED:
        assert np.array_equal(fa[k], fx[k]), ("stress", k)
        assert np.array_equal(fb[k], fy[k]), ("large", k)
    for run in (a, b, x, y):
        run.retire()


# ---- per field against the FP64 oracle at full size: one step from a state the faithful oracle grew
def _one_step_parity(ctx, state, label, bound=1e-5):
    o64 = O.OracleModel(state, fp64=True, threads=threads())
    o64.step(state.switches.dt, 1)
    ref = o64.fields()
    r = ctx.create(state)
    r.step(1)
    got = r.read()
    errs = field_errors(got, ref)
    thb = np.repeat(state.env.theta, state.grid.layer)
    errs["theta'"] = rel_l2(r.debug_read_set(0, "theta"), ref["theta"] - thb, FLOOR["theta'"])
    errs["precipitation"] = rel_l2(r.columns()["precipitation"], o64.get("precipitation"), 1e-9)
    st, oc = r.status(), o64.counters()
    print(f"\n{label}, one step vs FP64: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()) +
          f"; clipped {st['clipped']} (oracle {int(oc['clipped'])})")
    r.retire()
    bad = {k: v for k, v in errs.items() if not v <= bound}
    assert not bad, (label, bad)
    return st, oc, got, ref


def test_large_grid_one_step_per_field_against_fp64_oracle(ctx):
    """The large 80x64x50 grid (its layer spectrum in shared memory: the whole-layer 80-point warp transforms), a storm
    the faithful oracle grew for 300 steps from a 3 K bubble, one step on the device against the FP64 oracle: every
    field within 1e-5 relative L2."""
    state = developed_state(baseline_run(create_grid(LARGE_GRID), seed=5, bubble=3.0), 300)
    _one_step_parity(ctx, state, "large 80x64x50 after 300 steps")


def test_stress_grid_one_step_per_field_against_fp64_oracle(ctx):
    """The 320x256x80 stress grid (the row-transform path of the spectral solves at its real size), 25 faithful-oracle
    steps from a 3 K bubble, one step on the device against the FP64 oracle: every field within 1e-5 relative L2."""
    state = developed_state(baseline_run(create_grid(STRESS_GRID), seed=6, bubble=3.0), 25)
    _one_step_parity(ctx, state, "stress 320x256x80 after 25 steps")


def test_wind_limits_clip_like_the_oracle(ctx):
    """clipWind (src/core/model.ts:1586-1595): jets beyond the limits planted in a developed storm (u = 200 m/s on two
    whole x rows, v = -170 m/s on a whole y column, both uniform along their own axis so the projection keeps them; w =
    150 m/s in a 4x4 column over the layers between 8 and 13.5 km), one step: every field within 1e-5 of the FP64 oracle, the
    clamped nodes at exactly +-120 / +-100, and the same clipped count as the oracle's."""
    state = developed_state(baseline_run(create_grid(DEFAULT_GRID), seed=42), 300)
    g = state.grid
    f = {k: v.copy() for k, v in state.fields.items()}
    zu = int(np.searchsorted(g.zs, 2000.0))
    for y in (5, 6):
        f["u"][zu * g.layer + y * g.nx: zu * g.layer + (y + 1) * g.nx] = 200.0
    zv = int(np.searchsorted(g.zs, 3000.0))
    f["v"][zv * g.layer + 30 + g.nx * np.arange(g.ny)] = -170.0
    levels = [z for z in range(g.nz) if 8000.0 <= g.zs[z] <= 13500.0]  # layers of 500-730 m: Courant below 1
    for z in levels:
        for y in range(12, 16):
            f["w"][z * g.layer + y * g.nx + 20: z * g.layer + y * g.nx + 24] = 150.0
    from meteolab_gb300.scenarios import RunSpec
    jets = RunSpec(g, state.env, state.switches, f, state.seed, "jets")
    st, oc, got, ref = _one_step_parity(ctx, jets, "planted jets")
    assert st["clipped"] > 0 and st["clipped"] == int(oc["clipped"])
    for k, lim in (("u", 120.0), ("v", 120.0), ("w", 100.0)):
        assert float(np.max(np.abs(got[k]))) == lim
        assert np.array_equal(np.abs(got[k]) == lim, np.abs(ref[k]) == lim), k


def test_moving_frame_one_step_against_fp64_oracle(ctx):
    """A domain moving over the ground (frame_u = 10, frame_v = -4 m/s): the wind relaxation and the sponge act on
    uEnv = env.u - frame and the surface drag on the ground-relative wind (src/core/model.ts:1179-1194, :1478, :1495).
    A storm grown 300 steps in that frame by the faithful oracle, one step on the device against the FP64 oracle."""
    from meteolab_gb300.scenarios import Switches
    sw = Switches(frame_u=10.0, frame_v=-4.0)
    state = developed_state(baseline_run(create_grid(DEFAULT_GRID), seed=43, switches=sw), 300)
    _one_step_parity(ctx, state, "moving frame (10, -4) m/s")


def test_regime_point_with_a_lid_one_step_against_fp64_oracle(ctx):
    """A point of the uneven batch's regime grid (a slider-profile sounding: the moisture / lapse-rate knob, the
    hodograph scaled to its shear, an elevated mixed layer's lid), grown 200 steps by the faithful oracle, one step on
    the device against the FP64 oracle."""
    from meteolab_gb300.scenarios import regime_runs
    specs = [s for s in regime_runs(create_grid(DEFAULT_GRID), create_grid(LARGE_GRID), n_small=8, n_large=0, seed=88)
             if s.meta["lid_k"] > 0 and s.meta["cape"] > 1500]
    assert specs, "no lidded point with CAPE above 1500 J/kg among the eight"
    spec = max(specs, key=lambda s: s.meta["shear"])
    state = developed_state(spec, 200)
    _one_step_parity(ctx, state, f"regime point {spec.label} (ML CAPE {spec.meta['cape']:.0f} J/kg, shear {spec.meta['shear']:.0f} m/s, "
                                 f"lid {spec.meta['lid_k']:.1f} K at {spec.meta['lid_km']:.1f} km)")
