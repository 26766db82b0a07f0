"""TEST INFRASTRUCTURE ONLY — the oracle of the storm's electric potential: a numpy restatement of the reference's
ElectricSolver (src/core/electric.ts:15-72). Imported by tests/ and bench.py's CPU leg; never by the product.

∇²φ = -ρ/ε0 at the grid nodes, φ = 0 on the ground and top levels, periodic in x and y: the interior levels'
right-hand side -ρ/ε0 (:36-37) is transformed by a 2-D DFT per level (the reference's HorizontalDFT; here numpy's real
FFT, which gives the same modes m <= nx/2, all n), each mode solves the stretched vertical tridiagonal with fixed ends
(:41-56, Thomas, the rows and pivots in the reference's order), and the inverse transform gives the interior potential
(:57-59). `field` is the centred-difference E = -∇φ (:64-71).
"""
from __future__ import annotations

import numpy as np

EPSILON0 = 8.8541878128e-12  # src/core/electric.ts:6


def mode_symbols(nx: int, ny: int, dx: float, dy: float) -> np.ndarray:
    """[ny][nx//2 + 1]: minus the eigenvalue of the 5-point horizontal Laplacian per mode (electric.ts:29)."""
    m = np.arange(nx // 2 + 1)
    n = np.arange(ny)
    return (4 * np.sin(np.pi * m / nx) ** 2 / (dx * dx))[None, :] + (4 * np.sin(np.pi * n / ny) ** 2 / (dy * dy))[:, None]


def solve(grid, rho: np.ndarray) -> np.ndarray:
    """The potential (V) of the node charge density rho (C/m³, n = nx*ny*nz values, node x + nx(y + ny z))."""
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    if nz < 3:
        raise ValueError("the electric solver needs an interior level")
    dzs, hz = np.asarray(grid.dzs, np.float64), np.asarray(grid.hz, np.float64)
    ni = nz - 2
    inner = -np.asarray(rho, np.float64).reshape(nz, ny, nx)[1:nz - 1] / EPSILON0
    spec = np.fft.rfft2(inner)                       # [ni][ny][mh + 1]
    lam = mode_symbols(nx, ny, grid.dx, grid.dy)
    cp = np.zeros((ni,) + lam.shape)
    d = np.zeros_like(spec)
    for j in range(ni):                              # rows j = levels k = j + 1 (electric.ts:45-51)
        k = j + 1
        lo, up = 1.0 / (hz[k] * dzs[k - 1]), 1.0 / (hz[k] * dzs[k])
        di = -lo - up - lam
        a = lo if j > 0 else 0.0
        c = up if j < ni - 1 else 0.0
        piv = di if j == 0 else di - a * cp[j - 1]
        cp[j] = c / piv
        d[j] = (spec[j] - (0.0 if j == 0 else a * d[j - 1])) / piv
    for j in range(ni - 2, -1, -1):                  # back substitution (:52-55)
        d[j] = d[j] - cp[j] * d[j + 1]
    phi = np.zeros((nz, ny, nx))
    phi[1:nz - 1] = np.fft.irfft2(d, s=(ny, nx))
    return phi.ravel()


def field(grid, phi: np.ndarray, x: int, y: int, z: int):
    """E = -∇φ (V/m) at node (x, y, z): centred, periodic in x and y, one-sided at the ground and top (:64-71)."""
    nx, ny, nz, layer = grid.nx, grid.ny, grid.nz, grid.nx * grid.ny
    zs = np.asarray(grid.zs, np.float64)

    def at(i, j, k):
        return phi[((i + nx) % nx) + ((j + ny) % ny) * nx + k * layer]
    ex = -(at(x + 1, y, z) - at(x - 1, y, z)) / (2 * grid.dx)
    ey = -(at(x, y + 1, z) - at(x, y - 1, z)) / (2 * grid.dy)
    lo, hi = max(0, z - 1), min(nz - 1, z + 1)
    return ex, ey, -(at(x, y, hi) - at(x, y, lo)) / (zs[hi] - zs[lo])
