"""The device step at the benchmark's full sizes (GPU), through size-independent properties: the large 80x64x50
domain and the 320x256x80 stress grid (its layer spectrum too wide for shared memory: the row-transform path of the
spectral solves), each grown from a warm bubble for 100 steps (the scope of the large and stress configurations):
every field finite, no wind clipped, the post-projection divergence before its FP32 rounding at rounding level (the
projection's own operators in FP64 on the velocities and the pressure the device returns), water conserved with the
rain gauge to the reference's 1e-4 (src/core/invariants.test.ts:84-94), and the run the same alone and batched."""
import numpy as np
import pytest

from parity import WATER, dual_divergence, pressure_gradient, water_total
from meteolab_gb300.grid import LARGE_GRID, STRESS_GRID, create_grid
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
    big = baseline_run(create_grid(STRESS_GRID), seed=6, bubble=2.0)
    small = baseline_run(create_grid(LARGE_GRID), seed=7)
    a = ctx.create(big)
    a.step(5)
    x, y = ctx.create(big), ctx.create(small)
    ctx.batch_step([x, y], 5)
    fa, fx = a.read(), x.read()
    for k in CARRIED:
        assert np.array_equal(fa[k], fx[k]), k
    for run in (a, x, y):
        run.retire()
