"""The reference's terrain tests that stand on terrain.ts alone (src/core/terrain.test.ts:10-45 and :178-198) on the
oracle (CPU): the hill, ridge and plateau heights, the cut-cell projection of a uniform wind over a hill, and the face
apertures of a ramp. They pin the oracle's restatement of terrain.ts (oracle/oracle_terrain.h) that the device's masked
projection is checked against. (The file's other cases run the whole model with terrain, which the device step does
not carry.)"""
import numpy as np

import pyoracle as O
from meteolab_gb300.grid import GridOptions, create_grid

DT = 3.0
GRID = create_grid(GridOptions(32, 24, 30, 38_400, 28_800, 15_000, bottom_spacing=100))


def close(a, b, digits):  # vitest toBeCloseTo
    return abs(a - b) < 10 ** -digits / 2


def hill_case(grid=GRID):
    """terrain.test.ts:23-27: a 1 km hill of 5 km half-width, rho0 = 1.2 exp(-z / 9 km), a uniform 10 m/s westerly."""
    rho = 1.2 * np.exp(-np.asarray(grid.zs) / 9000)
    h = O.terrain_heights(grid, "hill", 1, 5)
    n = grid.nx * grid.ny * grid.nz
    return rho, h, np.full(n, 10, np.float32), np.zeros(n, np.float32), np.zeros(n, np.float32)


def test_hill_ridge_and_plateau_heights():  # terrain.test.ts:10-21
    nx, ny = GRID.nx, GRID.ny
    hill = O.terrain_heights(GRID, "hill", 1, 5)
    top = float(hill.max())
    assert 800 < top <= 1000 and hill[0] < .15 * top
    ridge = O.terrain_heights(GRID, "ridge", .8, 4)
    for j in range(1, ny):
        assert close(float(ridge[nx // 2 + nx * j]), float(ridge[nx // 2]), 3)
    plateau = O.terrain_heights(GRID, "plateau", .5, 8)
    assert plateau[nx // 2 + nx * (ny // 2)] > 450 and plateau[0] < 50
    assert hill.min() == 0 and ridge.min() == 0 and plateau.min() == 0


def test_projects_a_uniform_wind_over_a_hill():  # terrain.test.ts:23-45
    rho, h, u, v, w = hill_case()
    nx, ny, layer = GRID.nx, GRID.ny, GRID.nx * GRID.ny
    solid = O.terrain_geometry(GRID, h)["solid"]
    u, v, w, p, before, after, iterations, residual, dropped = O.masked_project(GRID, rho, h, u, v, w, DT)
    assert 0 < iterations < 200 and residual <= 1e-6
    assert np.linalg.norm(after) / np.linalg.norm(before) < 1e-5
    assert (u[solid == 1] == 0).all() and (w[solid == 1] == 0).all()
    cy = ny // 2

    def ground(x):
        z = 0
        while solid[x + nx * cy + z * layer]:
            z += 1
        return x + nx * cy + z * layer

    for x in range(nx):
        k = ground(x)
        if GRID.zs[k // layer] <= h[x + nx * cy]:
            assert w[k] == 0
    up, down = ground(nx // 2 - 4) + layer, ground(nx // 2 + 3) + layer
    assert w[up] > .5 and w[down] < -.5


def test_face_apertures_add_up_to_the_open_height():  # terrain.test.ts:178-198
    nx, nz, layer = GRID.nx, GRID.nz, GRID.nx * GRID.ny
    hz = np.asarray(GRID.hz)
    level = np.arange(GRID.nx * GRID.ny * nz) // layer
    plain = O.terrain_geometry(GRID, np.zeros(layer, np.float32))
    assert (plain["ax"] == hz[level]).all() and (plain["ay"] == hz[level]).all() and not plain["solid"].any()
    ramp = (37 * (np.arange(layer) % nx)).astype(np.float32)
    geo = O.terrain_geometry(GRID, ramp)
    ax, ay, solid, lid = geo["ax"], geo["ay"], geo["solid"], GRID.zs[nz - 1]
    for c in range(layer - 1):
        if c % nx == nx - 1:
            continue
        assert close(ax[c::layer].sum(), lid - (float(ramp[c]) + float(ramp[c + 1])) / 2, 6)
        assert close(ay[c::layer].sum(), lid - float(ramp[c]), 6)
    i = np.arange(layer * nz)
    c = i % layer
    east = (c % nx + 1) % nx + (c // nx) * nx + (i // layer) * layer
    shut = (solid[i] == 1) | (solid[east] == 1)
    assert (ax[shut] == 0).all()


def test_node_heights_add_up_to_the_column_above_the_ground():
    """nodeHeights (terrain.ts:101-105): a column's control volumes reach from its ground to the lid, the ground node a
    cut cell of at least LEAST_SHARE of its level (solidMask :80-84), the solid nodes none."""
    layer, nz = GRID.nx * GRID.ny, GRID.nz
    h = O.terrain_heights(GRID, "hill", 1, 5)
    geo = O.terrain_geometry(GRID, h)
    heights, solid, levels = geo["heights"], geo["solid"], geo["levels"]
    hz = np.asarray(GRID.hz)
    for c in range(layer):
        column = heights[c::layer]
        assert abs(column.sum() - (GRID.zs[nz - 1] - float(h[c]))) < 1e-9 * GRID.zs[nz - 1]
        g = levels[c]
        assert (solid[c::layer][:g] == 1).all() and not solid[c::layer][g:].any()
        assert (column[:g] == 0).all() and column[g] >= .2 * hz[g] - 1e-9
    assert levels.max() > 2 and (geo["slope"] >= 1).all() and geo["slope"].max() > 1.005


def test_a_flat_ground_projects_as_without_terrain():
    """MaskedProjection.project without terrain (terrain.ts:305, flat :336-339): the flat spectral projection, no
    iterations, the same velocities as the pressure projection."""
    rho, _, u, v, w = hill_case()
    rng = np.random.default_rng(3)
    u = (u + rng.normal(0, 1, u.size)).astype(np.float32)
    w = rng.normal(0, .5, w.size).astype(np.float32)
    layer = GRID.nx * GRID.ny
    flat = np.zeros(layer, np.float32)
    mu, mv, mw, p, before, after, iterations, residual, dropped = O.masked_project(GRID, rho, flat, u, v, w, DT)
    assert iterations == 0 and not dropped.any()
    w0 = w.copy()
    w0[:layer] = 0
    w0[-layer:] = 0
    pu, pv, pw = u.copy(), v.copy(), w0.copy()
    cells = layer * (GRID.nz - 1)
    d0, d1, pp = np.zeros(cells), np.zeros(cells), np.zeros(cells)
    args, keep = O.grid_args(GRID)
    O.lib().orc_pressure_project(*args, O.dp(O.f64(rho)), O.fp(pu), O.fp(pv), O.fp(pw), DT, O.dp(d0), O.dp(d1), O.dp(pp))
    assert np.array_equal(mu, pu) and np.array_equal(mv, pv) and np.array_equal(mw, pw) and np.array_equal(p, pp)


def schar_case():
    """terrain.test.ts:200-206: a 96 x 4 x 40 grid (48 x 2 x 15 km), a Schar ridge 100 m high (5 km envelope, 4 km
    waves), a uniform 10 m/s westerly."""
    g = create_grid(GridOptions(96, 4, 40, 48_000, 2_000, 15_000, bottom_spacing=100))
    rho = 1.2 * np.exp(-np.asarray(g.zs) / 9000)
    return g, rho, O.terrain_heights(g, "schar", .1, 5, wavelength=4)


def test_the_transport_sees_the_ridge_the_projection_sees():  # terrain.test.ts:200-226
    g, rho, h = schar_case()
    n, layer = g.nx * g.ny * g.nz, g.nx * g.ny
    U = np.full(n, 10, np.float32)
    zero = np.zeros(n, np.float32)
    u, v, w, *_ = O.masked_project(g, rho, h, U, zero, zero, 1.0)
    mx, my, mz, div, iterations, residual = O.masked_faces(g, rho, h, U, zero, zero)
    assert 0 < iterations < 400 and residual <= 1e-10
    for height in (1400, 2200, 3200):
        z = next(k for k, q in enumerate(g.zs) if q >= height)
        node = (w[z * layer:(z + 1) * layer].astype(float) + w[(z + 1) * layer:(z + 2) * layer]) / 2
        face = mz[z * layer:(z + 1) * layer] / ((rho[z] + rho[z + 1]) / 2)
        ratio = float(face @ node) / float(node @ node)
        assert (node @ node) > 0 and .98 < ratio < 1.03


def test_the_faces_into_the_ground_are_shut_and_the_rest_divergence_free():
    """setVelocityMasked (advection.ts:115-153) over a hill: no flux through a face next to a solid node, and the faces'
    divergence over the node heights down to the tolerance of the first (the water cannot cross the ground)."""
    rho, h, u, v, w = hill_case()
    g = GRID
    n, layer, nx = g.nx * g.ny * g.nz, g.nx * g.ny, g.nx
    rng = np.random.default_rng(5)
    w = rng.normal(0, 1, n).astype(np.float32)
    solid = O.terrain_geometry(g, h)["solid"]
    mx, my, mz, div, iterations, residual = O.masked_faces(g, rho, h, u, v, w)
    assert iterations > 0 and residual <= 1e-10
    i = np.arange(n)
    c = i % layer
    east = (c % nx + 1) % nx + (c // nx) * nx + (i // layer) * layer
    north = c % nx + ((c // nx + 1) % g.ny) * nx + (i // layer) * layer
    up = np.minimum(i + layer, n - 1)
    assert (mx[(solid == 1) | (solid[east] == 1)] == 0).all() and (my[(solid == 1) | (solid[north] == 1)] == 0).all()
    assert (mz[(solid == 1) | (solid[up] == 1) | (i >= n - layer)] == 0).all()
    fluid = solid == 0
    faces0 = O.masked_faces(g, rho, h, u, v, w, max_iterations=0)
    assert np.abs(div[fluid]).max() < 1e-7 * np.abs(faces0[3][fluid]).max()
