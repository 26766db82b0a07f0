"""The terrain's masked projection on the device (sg_masked_*, the reference's MaskedProjection, src/core/terrain.ts:168-363)
against the oracle and the reference's own test of it (src/core/terrain.test.ts:23-45), through the C ABI (GPU).

Tolerances: both solve in FP64 to the same relative residual (1e-6) along the same conjugate-gradient path; they differ
by rounding only (the device sums its DFTs directly and its dot products by blocks, the oracle by FFT and in order),
so the iterations agree to one and the projected winds to 1e-5 of their norm (rounding, then FP32 stores). The flat
ground is the plain spectral projection, to FP32 rounding.
"""
import numpy as np
import pytest

import pyoracle as O
from meteolab_gb300.grid import DEFAULT_GRID, GridOptions, create_grid

pytestmark = pytest.mark.gpu

DT = 3.0
TEST_GRID = create_grid(GridOptions(32, 24, 30, 38_400, 28_800, 15_000, bottom_spacing=100))


@pytest.fixture(scope="module")
def ctx():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import Context
    c = Context()
    yield c
    c.close()


def density(grid):
    return 1.2 * np.exp(-np.asarray(grid.zs) / 9000)


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def both(ctx, grid, ground, u, v, w, pressure, tolerance=1e-6, max_iterations=200):
    """The device's projection and the oracle's of the same winds and first guess."""
    from meteolab_gb300.runtime import MaskedProjection
    m = MaskedProjection(ctx, grid, density(grid), ground, tolerance, max_iterations)
    du, dv, dw, dp = u.copy(), v.copy(), w.copy(), pressure.copy()
    m.project(du, dv, dw, DT, dp)
    ref = O.masked_project(grid, density(grid), ground, u, v, w, DT, pressure, tolerance, max_iterations)
    return m, (du, dv, dw, dp), ref


def test_a_uniform_wind_over_a_hill(ctx):  # terrain.test.ts:23-45, on the device
    from meteolab_gb300.runtime import terrain_geometry, terrain_heights
    g = TEST_GRID
    nx, ny, layer, n = g.nx, g.ny, g.nx * g.ny, g.nx * g.ny * g.nz
    h = terrain_heights({"kind": "hill", "height": 1, "width": 5}, g)
    solid = terrain_geometry(g, h)["solid"]
    u, v, w = np.full(n, 10, np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32)
    m, (du, dv, dw, dp), ref = both(ctx, g, h, u, v, w, np.zeros(layer * (g.nz - 1)))
    ru, rv, rw, rp, before, after, iterations, residual, dropped = ref
    # The reference's assertions on the device's result.
    masked = [a.copy() for a in (u, v, w)]
    m.mask(*masked)
    b0, b1 = m.divergence(*masked), m.divergence(du, dv, dw)
    assert 0 < m.iterations < 200 and m.residual <= 1e-6
    assert np.linalg.norm(b1) / np.linalg.norm(b0) < 1e-5
    assert (du[solid == 1] == 0).all() and (dw[solid == 1] == 0).all()
    cy = ny // 2

    def ground(x):
        z = 0
        while solid[x + nx * cy + z * layer]:
            z += 1
        return x + nx * cy + z * layer

    for x in range(nx):
        k = ground(x)
        if g.zs[k // layer] <= h[x + nx * cy]:
            assert dw[k] == 0
    assert dw[ground(nx // 2 - 4) + layer] > .5 and dw[ground(nx // 2 + 3) + layer] < -.5
    # Against the oracle.
    assert abs(m.iterations - iterations) <= 1
    assert rel(du, ru) < 1e-5 and rel(dv, rv) < 1e-5 and rel(dw, rw) < 1e-5 and rel(dp, rp) < 1e-5
    assert rel(b0, before) < 1e-9 and np.array_equal(m.dropped, dropped)


@pytest.mark.parametrize("form", [("plateau", .5, 8, {}), ("schar", .4, 5, {"wavelength": 4}), ("ridge", 1.2, 3, {"heading": 60})],
                         ids=["plateau", "schar", "ridge60"])
def test_storm_winds_and_a_first_guess_match_the_oracle(ctx, form):
    """Random winds over other forms on the standard 40x32x50 grid, a non-zero first-guess pressure (the stages keep
    the last one); the second projection of the same object (its graph replayed) gives the same as a fresh one."""
    from meteolab_gb300.runtime import terrain_heights
    g = create_grid(DEFAULT_GRID)
    kind, height, width, extra = form
    h = terrain_heights(dict(kind=kind, height=height, width=width, **extra), g)
    n, cells = g.nx * g.ny * g.nz, g.nx * g.ny * (g.nz - 1)
    rng = np.random.default_rng(11)
    u = (12 + rng.normal(0, 3, n)).astype(np.float32)
    v = rng.normal(0, 3, n).astype(np.float32)
    w = rng.normal(0, 1, n).astype(np.float32)
    p0 = rng.normal(0, 20, cells)
    m, (du, dv, dw, dp), ref = both(ctx, g, h, u, v, w, p0)
    ru, rv, rw, rp, before, after, iterations, residual, dropped = ref
    assert abs(m.iterations - iterations) <= 1 and m.iterations > 0
    assert rel(du, ru) < 1e-5 and rel(dv, rv) < 1e-5 and rel(dw, rw) < 1e-5 and rel(dp, rp) < 1e-5
    again = [a.copy() for a in (u, v, w)] + [p0.copy()]
    m.project(*again[:3], DT, again[3])
    assert all(np.array_equal(x, y) for x, y in zip(again, (du, dv, dw, dp)))


def test_flat_ground_is_the_plain_projection(ctx):
    """No terrain at all (terrain.ts:305, :336-339): the flat spectral projection, no iterations."""
    g = TEST_GRID
    n, layer = g.nx * g.ny * g.nz, g.nx * g.ny
    rng = np.random.default_rng(3)
    u = (10 + rng.normal(0, 1, n)).astype(np.float32)
    v = rng.normal(0, 1, n).astype(np.float32)
    w = rng.normal(0, .5, n).astype(np.float32)
    m, (du, dv, dw, dp), ref = both(ctx, g, np.zeros(layer, np.float32), u, v, w, np.zeros(layer * (g.nz - 1)))
    ru, rv, rw, rp = ref[:4]
    assert m.iterations == 0 and ref[6] == 0
    assert np.abs(du - ru).max() < 1e-5 and np.abs(dv - rv).max() < 1e-5 and np.abs(dw - rw).max() < 1e-5
    assert rel(dp, rp) < 1e-10


def test_calm_air_and_a_short_solve(ctx):
    """Calm air has nothing to project (terrain.ts:309: no iterations, the first guess kept); three iterations at most
    stop at three, with the oracle's residual."""
    from meteolab_gb300.runtime import terrain_heights
    g = TEST_GRID
    n, cells = g.nx * g.ny * g.nz, g.nx * g.ny * (g.nz - 1)
    h = terrain_heights({"kind": "hill", "height": 1, "width": 5}, g)
    zero = np.zeros(n, np.float32)
    p0 = np.linspace(-1, 1, cells)
    m, (du, dv, dw, dp), ref = both(ctx, g, h, zero, zero, zero, p0)
    assert m.iterations == 0 and m.residual == 0 and ref[6] == 0
    assert not du.any() and not dv.any() and not dw.any() and np.array_equal(dp, p0)
    u = np.full(n, 10, np.float32)
    m, (du, dv, dw, dp), ref = both(ctx, g, h, u, zero, zero, np.zeros(cells), max_iterations=3)
    assert m.iterations == 3 and ref[6] == 3
    assert abs(m.residual - ref[7]) < 1e-6 * ref[7] and rel(dw, ref[2]) < 1e-5


def faces_both(ctx, grid, ground, u, v, w, **kw):
    from meteolab_gb300.runtime import TerrainFaces
    f = TerrainFaces(ctx, grid, density(grid), ground, **kw)
    mine = f.set_velocity_masked(u, v, w)
    ref = O.masked_faces(grid, density(grid), ground, u, v, w, **kw)
    return f, mine, ref


def test_transport_faces_over_a_hill_match_the_oracle(ctx):
    """setVelocityMasked (advection.ts:115-153) on the device against the oracle: a westerly with random vertical
    motion over the hill; the faces into the ground shut, the fluid nodes' divergence at the solve's tolerance."""
    from meteolab_gb300.runtime import terrain_geometry, terrain_heights
    g = TEST_GRID
    n, layer, nx = g.nx * g.ny * g.nz, g.nx * g.ny, g.nx
    h = terrain_heights({"kind": "hill", "height": 1, "width": 5}, g)
    rng = np.random.default_rng(5)
    u = np.full(n, 10, np.float32)
    v = np.zeros(n, np.float32)
    w = rng.normal(0, 1, n).astype(np.float32)
    f, (mx, my, mz, div), (rmx, rmy, rmz, rdiv, iterations, residual) = faces_both(ctx, g, h, u, v, w)
    assert abs(f.iterations - iterations) <= 1 and f.residual <= 1e-10
    assert rel(mx, rmx) < 1e-8 and rel(my, rmy) < 1e-8 and rel(mz, rmz) < 1e-8
    solid = terrain_geometry(g, h)["solid"]
    i = np.arange(n)
    c = i % layer
    east = (c % nx + 1) % nx + (c // nx) * nx + (i // layer) * layer
    assert (mx[(solid == 1) | (solid[east] == 1)] == 0).all()
    fluid = solid == 0
    assert np.abs(div[fluid]).max() < 1e-6 * np.abs(rmz).max() / min(g.hz)


def test_the_transport_sees_the_ridge_the_projection_sees_on_the_device(ctx):  # terrain.test.ts:200-226
    from meteolab_gb300.runtime import MaskedProjection, terrain_heights
    g = create_grid(GridOptions(96, 4, 40, 48_000, 2_000, 15_000, bottom_spacing=100))
    h = terrain_heights({"kind": "schar", "height": .1, "width": 5, "wavelength": 4}, g)
    n, layer, rho = g.nx * g.ny * g.nz, g.nx * g.ny, density(g)
    u, v, w = np.full(n, 10, np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32)
    m = MaskedProjection(ctx, g, rho, h)
    m.project(u, v, w, 1.0, np.zeros(layer * (g.nz - 1)))
    f, (mx, my, mz, div), ref = faces_both(ctx, g, h, np.full(n, 10, np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32))
    for height in (1400, 2200, 3200):
        z = next(k for k, q in enumerate(g.zs) if q >= height)
        node = (w[z * layer:(z + 1) * layer].astype(float) + w[(z + 1) * layer:(z + 2) * layer]) / 2
        face = mz[z * layer:(z + 1) * layer] / ((rho[z] + rho[z + 1]) / 2)
        assert (node @ node) > 0 and .98 < float(face @ node) / float(node @ node) < 1.03
    assert rel(mz, ref[2]) < 1e-8


def test_transport_faces_short_solve_and_calm_air(ctx):
    """Three iterations at most stop at three with the oracle's residual; calm air has nothing to project."""
    from meteolab_gb300.runtime import terrain_heights
    g = TEST_GRID
    n = g.nx * g.ny * g.nz
    h = terrain_heights({"kind": "plateau", "height": .5, "width": 8}, g)
    zero = np.zeros(n, np.float32)
    f, mine, ref = faces_both(ctx, g, h, zero, zero, zero)
    assert f.iterations == 0 and f.residual == 0 and ref[4] == 0 and not any(a.any() for a in mine)
    u = np.full(n, 10, np.float32)
    f, mine, ref = faces_both(ctx, g, h, u, zero, zero, max_iterations=3)
    assert f.iterations == 3 and ref[4] == 3 and abs(f.residual - ref[5]) < 1e-6 * ref[5] and rel(mine[2], ref[2]) < 1e-8
