"""Shared parity helpers of the tests: metrics and oracle-made states (the oracle is the checker only)."""
from __future__ import annotations

import os
from typing import Dict

import numpy as np

import pyoracle as O
from meteolab_gb300.scenarios import CARRIED, RunSpec

# Absolute floors of the relative L2 error for fields that can be (near) zero: ||a - b|| / max(||b||, floor sqrt(N)).
FLOOR = {"rain": 1e-8, "snow": 1e-8, "graupel": 1e-8, "hail": 1e-8, "cloud": 1e-8, "ice": 1e-8, "q": 1e-8,
         "iceNumber": 1.0, "cold": 1e-4, "u": 1e-3, "v": 1e-3, "w": 1e-3, "theta": 1e-3, "theta'": 1e-3}


def rel_l2(a, b, floor: float = 0.0) -> float:
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    den = max(float(np.linalg.norm(b)), floor * np.sqrt(b.size))
    num = float(np.linalg.norm(a - b))
    return 0.0 if num == 0.0 else num / den


def field_errors(got: Dict[str, np.ndarray], ref: Dict[str, np.ndarray], names=CARRIED) -> Dict[str, float]:
    return {k: rel_l2(got[k], ref[k], FLOOR.get(k, 0.0)) for k in names if k in got and k in ref}


def threads() -> int:
    return int(os.environ.get("SG_ORACLE_THREADS", "0")) or (os.cpu_count() or 1)


def developed_state(spec: RunSpec, steps: int) -> RunSpec:
    """The oracle's (faithful) state after `steps` steps, as a new run spec: a storm with condensate and rain."""
    m = O.OracleModel(spec, threads=threads())
    m.step(spec.switches.dt, steps)
    fields = {k: m.get(k).astype(np.float32) for k in CARRIED}
    return RunSpec(spec.grid, spec.env, spec.switches, fields, spec.seed, spec.label + f"+{steps}")


# ---- invariants of the reference's tests (src/core/fixtures.ts, src/core/pressure.ts)
WATER = ("q", "cloud", "ice", "rain", "snow", "graupel", "hail")


def level_mean(a, grid, z):
    """Horizontal mean of a field at level z (levelMean, src/core/fixtures.ts:33-38)."""
    return float(np.mean(np.asarray(a[z * grid.layer:(z + 1) * grid.layer], np.float64)))


def water_total(fields, precipitation, spec):
    """Total water in the air (mixing ratios weighted by rho0 h) plus what reached the ground, kg per m2 of ground
    (totalWater, src/core/fixtures.ts:44-56)."""
    g = spec.grid
    total = 0.0
    for z in range(g.nz):
        sl = slice(z * g.layer, (z + 1) * g.layer)
        level = sum(float(np.sum(np.asarray(fields[k][sl], np.float64))) for k in WATER)
        total += g.hz[z] * spec.env.rho[z] * level / g.layer
    return total + float(np.sum(np.asarray(precipitation, np.float64))) / g.layer


def dual_divergence(u, v, w, grid, rho):
    """Dual-cell divergence of rho0 u from the 8 corner nodes, FP64 (PressureSolver.divergence with dt = 1,
    src/core/pressure.ts:50-66)."""
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    U, V, W = (np.asarray(a, np.float64).reshape(nz, ny, nx) for a in (u, v, w))
    sx = lambda a: np.roll(a, -1, axis=2)
    sy = lambda a: np.roll(a, -1, axis=1)
    lo, hi = slice(0, nz - 1), slice(1, nz)
    r0 = (np.asarray(rho[:-1], np.float64) / 4)[:, None, None]
    r1 = (np.asarray(rho[1:], np.float64) / 4)[:, None, None]
    dz = np.asarray(grid.dzs[:nz - 1], np.float64)[:, None, None]
    ddx = (r0 * (sx(U)[lo] + sx(sy(U))[lo] - U[lo] - sy(U)[lo]) + r1 * (sx(U)[hi] + sx(sy(U))[hi] - U[hi] - sy(U)[hi])) / grid.dx
    ddy = (r0 * (sy(V)[lo] + sx(sy(V))[lo] - V[lo] - sx(V)[lo]) + r1 * (sy(V)[hi] + sx(sy(V))[hi] - V[hi] - sx(V)[hi])) / grid.dy
    ddz = (r1 * (W[hi] + sx(W)[hi] + sy(W)[hi] + sx(sy(W))[hi]) - r0 * (W[lo] + sx(W)[lo] + sy(W)[lo] + sx(sy(W))[lo])) / dz
    return ddx + ddy + ddz


def pressure_gradient(p, grid):
    """G p at the nodes from the dual-cell pressure (nx*ny*(nz-1), cell k between nodes k and k+1), FP64: the
    gradient of PressureSolver.correct (src/core/pressure.ts:69-92) - x and y from the four cells around each of the
    two neighbouring layers weighted by the spacings, z between the cell layers below and above; none at the ground and
    the top for z."""
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    P = np.asarray(p, np.float64).reshape(nz - 1, ny, nx)
    hz, dzs = np.asarray(grid.hz, np.float64), np.asarray(grid.dzs, np.float64)
    sx = lambda a: np.roll(a, 1, axis=2)   # the cell at x - 1
    sy = lambda a: np.roll(a, 1, axis=1)   # at y - 1
    k = np.arange(nz)
    lo, hi = P[np.maximum(0, k - 1)], P[np.minimum(nz - 2, k)]
    wlo = np.where(k > 0, dzs[np.maximum(0, k - 1)] / hz, 0.0)[:, None, None]
    whi = np.where(k < nz - 1, dzs[np.minimum(nz - 2, k)] / hz, 0.0)[:, None, None]
    dx4 = lambda a: (sy(a) - sx(sy(a))) + (a - sx(a))      # (x, jm) - (im, jm) + (x, j0) - (im, j0)
    dy4 = lambda a: (sx(a) - sx(sy(a))) + (a - sy(a))      # (im, j0) - (im, jm) + (x, j0) - (x, jm)
    gx = (wlo * dx4(lo) + whi * dx4(hi)) * (0.25 / grid.dx)
    gy = (wlo * dy4(lo) + whi * dy4(hi)) * (0.25 / grid.dy)
    c4 = lambda a: a + sx(a) + sy(a) + sx(sy(a))
    gz = np.zeros((nz, ny, nx))
    kk = np.arange(1, nz - 1)
    gz[kk] = (c4(P[kk]) - c4(P[kk - 1])) * (0.25 / hz[kk])[:, None, None]
    return gx.ravel(), gy.ravel(), gz.ravel()
