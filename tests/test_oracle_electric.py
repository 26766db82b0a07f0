"""The reference's electric-field tests (src/core/electric.test.ts) on the oracle of ElectricSolver (CPU).

These pin the oracle (oracle/electric.py) that the device solver is checked against: the discrete Laplacian of the
solution gives back -rho/eps0 to 1e-9 on a uniform and a stretched grid, a charged layer gives the parallel-plate
field above and below it, and a point charge gives Coulomb's field with its images in the ground and the top.
"""
import math
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle"))
import electric as E  # noqa: E402
from meteolab_gb300.grid import GridOptions, create_grid  # noqa: E402


def park_miller(seed):
    """The test's generator: seed = seed * 16807 mod (2^31 - 1), value seed / (2^31 - 1) - 0.5 (electric.test.ts:10)."""
    while True:
        seed = (seed * 16807) % 2147483647
        yield seed / 2147483647 - .5


def laplacian_residual(grid, rho, phi):
    """max |discrete Laplacian of phi + rho/eps0| over the interior nodes, relative to max |rho/eps0| (:13-20)."""
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    p = phi.reshape(nz, ny, nx)
    dzs, hz = np.asarray(grid.dzs), np.asarray(grid.hz)
    k = np.arange(1, nz - 1)
    pk = p[1:nz - 1]
    lap = ((np.roll(pk, -1, 2) - 2 * pk + np.roll(pk, 1, 2)) / grid.dx ** 2 + (np.roll(pk, -1, 1) - 2 * pk + np.roll(pk, 1, 1)) / grid.dy ** 2
           + ((p[2:] - pk) / dzs[k][:, None, None] - (pk - p[:nz - 2]) / dzs[k - 1][:, None, None]) / hz[k][:, None, None])
    target = -rho.reshape(nz, ny, nx)[1:nz - 1] / E.EPSILON0
    return float(np.max(np.abs(lap - target)) / np.max(np.abs(target)))


def random_charge(grid, seed=7):
    g = park_miller(seed)
    return np.array([next(g) * 1e-9 for _ in range(grid.nx * grid.ny * grid.nz)])


def plate_grid():
    return create_grid(GridOptions(4, 4, 81, 4000.0, 4000.0, 20_000.0, None))


def plate_charge(grid):
    rho = np.zeros(grid.nx * grid.ny * grid.nz)
    for k in range(grid.nz):
        if 6000 <= grid.zs[k] <= 8000:
            rho[k * grid.nx * grid.ny:(k + 1) * grid.nx * grid.ny] = 1e-9
    return rho


def check_plate(grid, phi, field):
    """The field below and above a 1 nC/m3 layer between 6 and 8 km under a 20 km top (:24-37)."""
    sigma, h, H = 1e-9 * 9 * 250, 7000.0, 20_000.0
    below = field(grid, phi, 1, 1, 8)[2]
    above = field(grid, phi, 1, 1, 60)[2]
    assert abs(below / (-sigma * (H - h) / (H * E.EPSILON0)) - 1) < 5e-7
    assert abs(above / (sigma * h / (H * E.EPSILON0)) - 1) < 5e-7
    assert 160e3 < abs(below) < 170e3


def point_grid():
    return create_grid(GridOptions(120, 120, 41, 60_000.0, 60_000.0, 20_000.0, None))


def point_charge(grid):
    n, c, kc = grid.nx, grid.nx // 2, 12
    rho = np.zeros(grid.nx * grid.ny * grid.nz)
    rho[c + c * n + kc * grid.nx * grid.ny] = 1.0 / (grid.dx * grid.dy * grid.hz[kc])
    return rho


def check_point(grid, phi, field):
    """Coulomb's field of 1 C at 6 km with its images in the ground and the top and the periodic copies, 12 nodes
    away, within 2% (:40-64)."""
    c, kc = grid.nx // 2, 12

    def coulomb(x, y, z):
        ex = ey = ez = 0.0
        for px in (-1, 0, 1):
            for py in (-1, 0, 1):
                for m in range(-6, 7):
                    for zq, q in ((2 * m * 20_000 + 6000, 1.0), (2 * m * 20_000 - 6000, -1.0)):
                        rx, ry, rz = x - px * 60_000, y - py * 60_000, z - zq
                        r = math.sqrt(rx * rx + ry * ry + rz * rz)
                        f = q / (4 * math.pi * E.EPSILON0 * r ** 3)
                        ex += f * rx; ey += f * ry; ez += f * rz
        return ex, ey, ez

    for dxn, dyn, k in ((12, 0, kc), (0, -12, kc), (9, 9, kc), (0, 0, kc + 12), (12, 0, 2)):
        got = field(grid, phi, c + dxn, c + dyn, k)
        want = coulomb(dxn * grid.dx, dyn * grid.dy, grid.zs[k])
        err = math.dist(got, want) / math.hypot(*want)
        assert err < .02, (dxn, dyn, k, err)


def test_solves_the_discrete_poisson_equation_exactly():
    for bottom in (None, 150.0):
        grid = create_grid(GridOptions(12, 10, 18, 12 * 1200.0, 10 * 1100.0, 18_000.0, bottom))
        rho = random_charge(grid)
        phi = E.solve(grid, rho)
        assert laplacian_residual(grid, rho, phi) < 1e-9
        layer = grid.nx * grid.ny
        assert np.all(phi[:layer] == 0) and np.all(phi[-layer:] == 0)


def test_a_charged_layer_gives_the_parallel_plate_field():
    grid = plate_grid()
    check_plate(grid, E.solve(grid, plate_charge(grid)), E.field)


def test_a_point_charge_gives_coulomb_with_its_images():
    grid = point_grid()
    check_point(grid, E.solve(grid, point_charge(grid)), E.field)


@pytest.mark.parametrize("shape", [(4, 3, 7, 120.0), (5, 4, 3, None), (6, 5, 9, 80.0)])
def test_matches_a_dense_solve_of_the_same_equations(shape):
    """The oracle against a direct dense solve of the discrete equations it restates (electric.ts:13-19): the periodic
    5-point horizontal Laplacian plus the stretched vertical one at every interior node, phi = 0 on the ground and top."""
    nx, ny, nz, bottom = shape
    grid = create_grid(GridOptions(nx, ny, nz, nx * 900.0, ny * 1000.0, 4000.0, bottom))
    rng = np.random.default_rng(nx * 100 + nz)
    rho = rng.standard_normal(nx * ny * nz) * 1e-9
    layer, ni = nx * ny, nz - 2
    dzs, hz = np.asarray(grid.dzs), np.asarray(grid.hz)
    A = np.zeros((ni * layer, ni * layer))
    idx = lambda x, y, k: ((x % nx) + (y % ny) * nx) + (k - 1) * layer
    for k in range(1, nz - 1):
        lo, up = 1 / (hz[k] * dzs[k - 1]), 1 / (hz[k] * dzs[k])
        for y in range(ny):
            for x in range(nx):
                r = idx(x, y, k)
                for (xx, yy, c) in ((x + 1, y, 1 / grid.dx ** 2), (x - 1, y, 1 / grid.dx ** 2), (x, y + 1, 1 / grid.dy ** 2), (x, y - 1, 1 / grid.dy ** 2)):
                    A[r, idx(xx, yy, k)] += c
                A[r, r] -= 2 / grid.dx ** 2 + 2 / grid.dy ** 2 + lo + up
                if k - 1 >= 1:
                    A[r, idx(x, y, k - 1)] += lo
                if k + 1 <= nz - 2:
                    A[r, idx(x, y, k + 1)] += up
    b = -rho[layer:(nz - 1) * layer] / E.EPSILON0
    want = np.linalg.solve(A, b)
    got = E.solve(grid, rho)[layer:(nz - 1) * layer]
    assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))
