"""The oracle's per-run diagnostics pinned to the reference's own tests (CPU): countCores
(src/core/model.test.ts:25-31), the core vorticity of a rotating updraught against a vortex pair (:33-55), and the
swaths' fold onto the ground under a moving domain (src/ensemble/ensemble.test.ts:23-31). The same cases run through
the device in tests/test_gpu_diag.py."""
import dataclasses

import numpy as np
import pytest

import pyoracle as O
from meteolab_gb300.grid import DEFAULT_GRID, create_grid
from meteolab_gb300.scenarios import baseline_run


def model(grid_opts=DEFAULT_GRID, frame=(0.0, 0.0)):
    spec = baseline_run(create_grid(grid_opts), seed=1)
    if frame != (0.0, 0.0):
        spec = dataclasses.replace(spec, switches=dataclasses.replace(spec.switches, frame_u=frame[0], frame_v=frame[1]))
    return spec, O.OracleModel(spec, fp64=True, threads=1)


def cores_fields(grid):
    """model.test.ts:25-31: cloudy cores (w = 8 m/s, cloud 1e-3) at 2-6 km in two columns, one only at 0.3-1.2 km."""
    n, nx, layer = grid.n, grid.nx, grid.layer
    w, cloud = np.zeros(n), np.zeros(n)
    for (x, y, lo, hi) in ((5, 5, 2000, 6000), (25, 20, 2000, 6000), (15, 10, 300, 1200)):
        for k, z in enumerate(grid.zs):
            if lo <= z <= hi:
                w[x + nx * y + k * layer] = 8
                cloud[x + nx * y + k * layer] = 1e-3
    return {"w": w, "cloud": cloud, "ice": np.zeros(n)}


def vortex_fields(grid, vortices, cx=20, cy=16):
    """model.test.ts:35-50: a broad updraught at 1.5-6 km and Rankine vortices (zeta inside 2 km) at column offsets."""
    nx, ny, layer = grid.nx, grid.ny, grid.layer
    u, v, w = np.zeros(grid.n), np.zeros(grid.n), np.zeros(grid.n)
    for z, zz in enumerate(grid.zs):
        if zz < 1500 or zz > 6000:
            continue
        for y in range(ny):
            for x in range(nx):
                i = x + nx * y + z * layer
                ex, ny_ = (x - cx) * grid.dx, (y - cy) * grid.dy
                w[i] = 25 * np.exp(-(ex * ex + ny_ * ny_) / 5000 ** 2)
                for ox, zeta in vortices:
                    rx = ex - ox * grid.dx
                    r = np.hypot(rx, ny_)
                    speed = zeta / 2 * (r if r < 2000 else 2000 ** 2 / r)
                    if r > 0:
                        u[i] += -speed * ny_ / r
                        v[i] += speed * rx / r
    return {"u": u, "v": v, "w": w}


def test_counts_updraught_cores_by_height():
    spec, m = model()
    for k, a in cores_fields(spec.grid).items():
        m.set(k, a)
    assert m.diagnostics()["cores"] == 2


def test_tells_a_rotating_updraught_from_a_vortex_pair():
    spec, m = model()
    for k, a in vortex_fields(spec.grid, [(0, .02)]).items():
        m.set(k, a)
    m.update_rotation(1)
    meso, _ = m.rotation()
    for k, a in vortex_fields(spec.grid, [(-3, .02), (3, -.02)]).items():
        m.set(k, a)
    m.update_rotation(1)
    pair, _ = m.rotation()
    assert meso["coreZeta"] > .004
    assert pair["uh"] > 200 and pair["anticyclonic"] > 200
    assert abs(pair["coreZeta"]) < .002


def test_swaths_fold_onto_the_ground_under_a_moving_domain():
    # ensemble.test.ts:23-31: 4 x 2 columns of 1 km, the domain moved 2 km east (5 m/s for 400 s): column 1 lies over
    # ground column 3
    opts = dataclasses.replace(DEFAULT_GRID, nx=4, ny=2, nz=6, width=4000.0, depth=2000.0)
    spec, m = model(opts, frame=(5.0, 0.0))
    g = spec.grid
    u = np.zeros(g.n)
    u[1] = 10
    m.set("u", u)
    m.set("v", np.zeros(g.n))
    uh = np.zeros(g.layer)
    uh[1] = 300
    m.add_swaths(400.0, uh)
    gust, uhmax = m.swaths()
    assert uhmax[3] == 300 and gust[3] == 15 and gust[0] == 5
