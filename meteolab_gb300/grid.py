"""Model grid of the StormLab step: node levels, spacings, control-volume heights.

Restates ``createGrid``/``stretchRatio``/``DEFAULT_GRID``/``LARGE_GRID`` of the reference
(src/core/grid.ts:31-34, :91-121). Nodes are ``i = x + nx*(y + ny*z)`` (x fastest), periodic in x and y;
levels span ``0..height`` inclusive, stretched geometrically from ``bottom_spacing`` when it is given.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass(frozen=True)
class GridOptions:
    nx: int
    ny: int
    nz: int
    width: float
    depth: float
    height: float
    bottom_spacing: float | None = None


#: The standard domain, 48 x 36 km at 1.2 x 1.125 km, 50 levels stretched from 100 m to 18.9 km (src/core/grid.ts:31).
DEFAULT_GRID = GridOptions(40, 32, 50, 48_000.0, 36_000.0, 18_900.0, 100.0)
#: The large domain, 96 x 72 km at the same spacing (src/core/grid.ts:34).
LARGE_GRID = GridOptions(80, 64, 50, 96_000.0, 72_000.0, 18_900.0, 100.0)
#: The bandwidth stress grid: 320 x 256 columns at 300 m, 80 levels with the same stretching law.
STRESS_GRID = GridOptions(320, 256, 80, 96_000.0, 76_800.0, 18_900.0, 100.0)


def stretch_ratio(bottom: float, height: float, intervals: int) -> float:
    """Geometric ratio r with bottom*(r^m - 1)/(r - 1) = height, by bisection (src/core/grid.ts:91-97)."""
    if bottom * intervals >= height:
        return 1.0
    lo, hi = 1.0, 2.0
    while bottom * (hi ** intervals - 1) / (hi - 1) < height:
        hi *= 2
    for _ in range(100):
        mid = (lo + hi) / 2
        if bottom * (mid ** intervals - 1) / (mid - 1) < height:
            lo = mid
        else:
            hi = mid
    return (lo + hi) / 2


@dataclass
class Grid:
    """A built grid (src/core/grid.ts:99-121): levels ``zs``, spacings ``dzs`` (nz-1), control volumes ``hz``."""
    nx: int
    ny: int
    nz: int
    width: float
    depth: float
    height: float
    dx: float
    dy: float
    dz: float
    uniform: bool
    zs: np.ndarray = field(repr=False)
    dzs: np.ndarray = field(repr=False)
    hz: np.ndarray = field(repr=False)

    @property
    def n(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def layer(self) -> int:
        return self.nx * self.ny

    @property
    def options(self) -> GridOptions:
        return GridOptions(self.nx, self.ny, self.nz, self.width, self.depth, self.height,
                           None if self.uniform else float(self.dzs[0]))


def create_grid(options: GridOptions = DEFAULT_GRID) -> Grid:
    """Build the levels exactly as ``createGrid`` does (src/core/grid.ts:99-121)."""
    nx, ny, nz = options.nx, options.ny, options.nz
    if nx < 1 or ny < 1 or nz < 2:
        raise ValueError(f"grid needs nx, ny >= 1 and nz >= 2, got {nx}x{ny}x{nz}")
    dz = options.height / (nz - 1)
    zs = np.zeros(nz)
    if options.bottom_spacing is None:
        zs = np.array([z * dz for z in range(nz)], dtype=np.float64)
    else:
        r = stretch_ratio(options.bottom_spacing, options.height, nz - 1)
        for z in range(1, nz):
            zs[z] = zs[z - 1] + options.bottom_spacing * r ** (z - 1)
        top = zs[nz - 1]
        for z in range(1, nz):
            zs[z] *= options.height / top
    if options.bottom_spacing is None:
        dzs = np.full(nz - 1, dz)
    else:
        dzs = np.array([zs[k + 1] - zs[k] for k in range(nz - 1)], dtype=np.float64)
    hz = np.array([((dzs[k - 1] if k > 0 else 0.0) + (dzs[k] if k < nz - 1 else 0.0)) / 2 for k in range(nz)],
                  dtype=np.float64)
    return Grid(nx, ny, nz, options.width, options.depth, options.height, options.width / nx, options.depth / ny,
                dz, options.bottom_spacing is None, zs, dzs, hz)


def level_at(grid: Grid, height: float) -> float:
    """Fractional level index of a height (src/core/grid.ts:358-365)."""
    zs, nz = grid.zs, grid.nz
    if height <= 0:
        return 0.0
    if height >= zs[nz - 1]:
        return float(nz - 1)
    k = 0
    while zs[k + 1] < height:
        k += 1
    return k + (height - zs[k]) / (zs[k + 1] - zs[k])
