"""The storm's electric potential on the device (sg_electric_*, the reference's ElectricSolver) against the oracle and
the reference's own tests (src/core/electric.test.ts), through the C ABI (GPU).

Tolerances: both are FP64; the device sums its DFTs directly, the oracle by FFT, so the potentials agree to rounding
(1e-10 of the largest). The reference's tests keep their own bounds: the discrete Poisson equation to 1e-9, the
plate field to 5e-7, Coulomb's field within 2%.
"""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "oracle"))
import electric as E  # noqa: E402
from meteolab_gb300.grid import DEFAULT_GRID, GridOptions, create_grid  # noqa: E402
from test_oracle_electric import (check_plate, check_point, laplacian_residual, plate_charge, plate_grid, point_charge,  # noqa: E402
                                  point_grid, random_charge)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import Context
    c = Context()
    yield c
    c.close()


def solver(ctx, grid):
    from meteolab_gb300.runtime import ElectricSolver
    return ElectricSolver(ctx, grid)


def test_matches_the_oracle_on_the_standard_grid(ctx):
    """A storm-like charge on the standard 40x32x50 grid: a positive layer over a negative one, plus noise."""
    grid = create_grid(DEFAULT_GRID)
    rng = np.random.default_rng(3)
    z = np.repeat(np.asarray(grid.zs), grid.nx * grid.ny)
    rho = 1e-9 * (np.exp(-((z - 9000) / 1500) ** 2) - np.exp(-((z - 6000) / 1000) ** 2)) + 1e-11 * rng.standard_normal(z.size)
    s = solver(ctx, grid)
    got = s.solve(rho)
    want = E.solve(grid, rho)
    assert np.max(np.abs(got - want)) <= 1e-10 * np.max(np.abs(want))
    assert laplacian_residual(grid, rho, got) < 1e-9
    # a second solve on the same solver (its scratch reused) gives the same potential
    assert np.array_equal(s.solve(rho), got)
    s.close()


def test_solves_the_discrete_poisson_equation_exactly(ctx):
    for bottom in (None, 150.0):
        grid = create_grid(GridOptions(12, 10, 18, 12 * 1200.0, 10 * 1100.0, 18_000.0, bottom))
        rho = random_charge(grid)
        s = solver(ctx, grid)
        phi = s.solve(rho)
        assert laplacian_residual(grid, rho, phi) < 1e-9
        layer = grid.nx * grid.ny
        assert np.all(phi[:layer] == 0) and np.all(phi[-layer:] == 0)
        s.close()


def test_a_charged_layer_gives_the_parallel_plate_field(ctx):
    grid = plate_grid()
    s = solver(ctx, grid)
    check_plate(grid, s.solve(plate_charge(grid)), lambda g, phi, x, y, z: s.field(phi, x, y, z))
    s.close()


def test_a_point_charge_gives_coulomb_with_its_images(ctx):
    grid = point_grid()
    s = solver(ctx, grid)
    check_point(grid, s.solve(point_charge(grid)), lambda g, phi, x, y, z: s.field(phi, x, y, z))
    s.close()


def test_a_grid_without_interior_levels_is_refused(ctx):
    from meteolab_gb300.runtime import StormGpuError
    grid = create_grid(GridOptions(8, 8, 2, 8000.0, 8000.0, 1000.0, None))
    with pytest.raises(StormGpuError, match="needs an interior level"):
        solver(ctx, grid)


@pytest.mark.parametrize("shape", [(5, 4, 3, None), (4, 3, 7, 120.0), (7, 6, 9, 80.0), (1, 1, 6, None), (9, 2, 5, None)])
def test_small_and_odd_grids_match_the_oracle(ctx, shape):
    """Odd widths (no Nyquist column), a single interior level, a single column and two-row grids."""
    nx, ny, nz, bottom = shape
    grid = create_grid(GridOptions(nx, ny, nz, nx * 900.0, ny * 1000.0, 4000.0, bottom))
    rho = np.random.default_rng(nx * 100 + nz).standard_normal(nx * ny * nz) * 1e-9
    s = solver(ctx, grid)
    got = s.solve(rho)
    s.close()
    want = E.solve(grid, rho)
    assert np.max(np.abs(got - want)) <= 1e-10 * np.max(np.abs(want))
