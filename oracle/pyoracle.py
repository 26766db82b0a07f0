"""TEST INFRASTRUCTURE ONLY — ctypes front end of the oracle (the CPU restatement of the reference's StormLab step,
oracle/oracle_*.h). Imported by tests/, __graft_entry__.smoke() and bench.py's CPU legs; never by the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_lock = threading.Lock()
_lib = None

CARRIED = ("rain", "snow", "graupel", "hail", "u", "v", "w", "theta", "q", "cloud", "ice", "iceNumber", "cold")
EXTRA = {"precipitation": 100, "hailGround": 101, "hailSize": 102, "fallSpeed": 103, "snowFall": 104,
         "graupelFall": 105, "hailFall": 106, "condensate": 107}

_d = C.POINTER(C.c_double)
_f = C.POINTER(C.c_float)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (plain g++/OpenMP)."""
    sources = [os.path.join(HERE, n) for n in ("oracle.cpp", "oracle_core.h", "oracle_solvers.h", "oracle_model.h", "oracle_diag.h")]
    if force or not os.path.exists(LIB_PATH) or any(os.path.getmtime(s) > os.path.getmtime(LIB_PATH) for s in sources):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB_PATH)
            L.orc_create.restype = C.c_void_p
            L.orc_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                     _d, _d, _d, _d, _d, C.c_int]
            L.orc_destroy.argtypes = [C.c_void_p]
            L.orc_set_threads.argtypes = [C.c_void_p, C.c_int]
            L.orc_set_field.argtypes = [C.c_void_p, C.c_int, _d, C.c_long]
            L.orc_get_field.argtypes = [C.c_void_p, C.c_int, _d, C.c_long]
            L.orc_step.argtypes = [C.c_void_p, C.c_double, C.c_int]
            L.orc_step_part.argtypes = [C.c_void_p, C.c_double, C.c_int]
            L.orc_get_pressure.argtypes = [C.c_void_p, _d, C.c_long]
            L.orc_get_faces.argtypes = [C.c_void_p, _d, _d, _d, _d, C.c_long]
            L.orc_counters.argtypes = [C.c_void_p, _d]
            L.orc_update_rotation.argtypes = [C.c_void_p, C.c_double]
            L.orc_rotation.argtypes = [C.c_void_p, _d, _d]
            L.orc_set_persisted.argtypes = [C.c_void_p, C.c_double]
            L.orc_diagnostics.argtypes = [C.c_void_p, _d]
            L.orc_swaths.argtypes = [C.c_void_p, _f, _f]
            L.orc_add_swaths.argtypes = [C.c_void_p, C.c_double, _d]
            for name in ("orc_weno", "orc_upwind5"):
                getattr(L, name).restype = C.c_double
                getattr(L, name).argtypes = [C.c_double] * 5
            for name, nargs in (("orc_qsat", 2), ("orc_qsat_ice", 2), ("orc_fall_speed", 3), ("orc_snow_fall_speed", 3),
                                ("orc_graupel_fall_speed", 2), ("orc_hail_fall_speed", 2), ("orc_hail_max_diameter", 2),
                                ("orc_cooper", 1), ("orc_splintering", 1), ("orc_fragments", 1), ("orc_koenig", 2),
                                ("orc_plate_size", 1), ("orc_crystal_size", 3)):
                getattr(L, name).restype = C.c_double
                getattr(L, name).argtypes = [C.c_double] * nargs
            L.orc_cell.restype = C.c_double
            L.orc_cell.argtypes = [C.c_int, _f, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double]
            L.orc_microphysics.restype = C.c_double
            L.orc_microphysics.argtypes = [_f, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
            L.orc_microphysics64.restype = C.c_double
            L.orc_microphysics64.argtypes = [_d, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
            L.orc_fft.argtypes = [C.c_int, _d, _d, C.c_int]
            L.orc_hdft.argtypes = [C.c_int, C.c_int, C.c_int, _d, _d, _d, _d]
            grid_args = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _d, _d, _d]
            L.orc_pressure_project.argtypes = grid_args + [_d, _f, _f, _f, C.c_double, _d, _d, _d]
            L.orc_transport.argtypes = grid_args + [_d, _f, _f, _f, _f, C.c_double, C.c_int, C.c_int, _d, _d, _d, _d]
            L.orc_turbulence.argtypes = grid_args + [_d, _f, _f, _f, _f, _d, C.c_double, C.c_double, _f, _f, _d, C.c_int,
                                                     C.c_int, C.c_int, C.c_int, _d, _d, _d, _d, _f, _d, C.c_double, C.c_int]
            _lib = L
    return _lib


def dp(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(_d)


def fp(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data_as(_f)


def f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def grid_args(grid):
    zs, dzs, hz = f64(grid.zs), f64(grid.dzs), f64(grid.hz)
    return (grid.nx, grid.ny, grid.nz, grid.dx, grid.dy, grid.dz, grid.height, dp(zs), dp(dzs), dp(hz)), (zs, dzs, hz)


def switch_vector(sw, grid, slabs: int = 1) -> np.ndarray:
    """The oracle's 20 switches from a ``meteolab_gb300.scenarios.Switches``."""
    return np.array([sw.coriolis, sw.wind_relaxation, sw.sponge_rate, sw.sponge_start, sw.cs, sw.drag_cd(grid),
                     sw.frame_u, sw.frame_v, sw.loading, sw.evaporation, sw.rain_formation, sw.anisotropic,
                     sw.vertical_dz, sw.durran_klemp, sw.pressure_in_stages, 1, 0.0, 0.0, 1, slabs], dtype=np.float64)


class OracleModel:
    """The oracle's model on one run (faithful: FP32 storage, FP64 arithmetic; ``fp64``: pure FP64)."""

    def __init__(self, spec, fp64: bool = False, threads: int = 0, slabs: int = 1):
        L = lib()
        g = spec.grid
        self.grid, self.spec = g, spec
        env = spec.env
        env7 = f64(np.concatenate([env.p, env.exner, env.theta, env.q, env.u, env.v, env.rho]))
        sw = switch_vector(spec.switches, g, slabs)
        args, keep = grid_args(g)
        threads = threads or os.cpu_count() or 1
        self.h = L.orc_create(1 if fp64 else 0, *args[:7], args[7], args[8], args[9], dp(env7), dp(sw), threads)
        self._keep = (keep, env7, sw)
        for name, arr in spec.fields.items():
            self.set(name, arr)

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().orc_destroy(h)
            self.h = None

    def set_threads(self, threads: int):
        lib().orc_set_threads(self.h, threads)

    def _id(self, name: str) -> int:
        return CARRIED.index(name) if name in CARRIED else EXTRA[name]

    def set(self, name: str, values: np.ndarray):
        a = f64(values).ravel()
        if lib().orc_set_field(self.h, self._id(name), dp(a), a.size):
            raise ValueError(f"bad field {name}")

    def get(self, name: str) -> np.ndarray:
        n = self.grid.layer if name in ("precipitation", "hailGround", "hailSize") else self.grid.n
        out = np.empty(n)
        if lib().orc_get_field(self.h, self._id(name), dp(out), n):
            raise ValueError(f"bad field {name}")
        return out

    def fields(self) -> Dict[str, np.ndarray]:
        return {k: self.get(k) for k in CARRIED}

    def step(self, dt: float, steps: int = 1):
        lib().orc_step(self.h, dt, steps)

    def step_part(self, dt: float, part: int):
        lib().orc_step_part(self.h, dt, part)

    def pressure(self) -> np.ndarray:
        out = np.empty(self.grid.nx * self.grid.ny * (self.grid.nz - 1))
        lib().orc_get_pressure(self.h, dp(out), out.size)
        return out

    def faces(self):
        n = self.grid.n
        mx, my, mz, dv = np.empty(n), np.empty(n), np.empty(n), np.empty(n)
        lib().orc_get_faces(self.h, dp(mx), dp(my), dp(mz), dp(dv), n)
        return mx, my, mz, dv

    def counters(self) -> Dict[str, float]:
        out = np.empty(7)
        lib().orc_counters(self.h, dp(out))
        return dict(clipped=out[0], negativeFilled=out[1], condensed=out[2], evaporated=out[3],
                    rainEvaporated=out[4], surface=out[5], time=out[6])


ROTATION = ("uh", "x", "y", "anticyclonic", "persisted", "uh01", "uh03", "low", "coreZeta", "coreUH", "coreAnti")
DIAGNOSTICS = ("updraft", "downdraft", "rainRate", "rainTotal", "cloudTop", "thermalTop", "maxCloud", "coldMax", "cores",
               "outflow", "outflowLow", "gust", "hail", "clipped")


def _rotation(self):
    """The rotation tracking's state after the last step (updateRotation) and the UH column."""
    out, col = np.empty(len(ROTATION)), np.empty(self.grid.layer)
    lib().orc_rotation(self.h, dp(out), dp(col))
    return dict(zip(ROTATION, out)), col


def _update_rotation(self, dt: float):
    lib().orc_update_rotation(self.h, dt)


def _diagnostics(self):
    out = np.empty(len(DIAGNOSTICS))
    lib().orc_diagnostics(self.h, dp(out))
    return dict(zip(DIAGNOSTICS, out))


def _swaths(self):
    g, u = np.empty(self.grid.layer, np.float32), np.empty(self.grid.layer, np.float32)
    lib().orc_swaths(self.h, g.ctypes.data_as(_f), u.ctypes.data_as(_f))
    return g, u


OracleModel.rotation = _rotation
OracleModel.update_rotation = _update_rotation
OracleModel.diagnostics = _diagnostics
def _add_swaths(self, time: float, uh_column):
    lib().orc_add_swaths(self.h, time, dp(np.ascontiguousarray(uh_column, np.float64)))


OracleModel.swaths = _swaths
OracleModel.add_swaths = _add_swaths


def cell(which: str, values: Dict[str, float], exner=1.0, p=1e5, rho=1.0, dt=1.0, aux=0.0):
    """Run one of the reference's per-cell processes on float32 cells; returns (result, cell after)."""
    names = ("theta", "q", "cloud", "ice", "snow", "rain", "graupel", "hail", "number")
    v = np.array([values.get(n, 0.0) for n in names], dtype=np.float32)
    code = {"rain": 0, "satadjust": 1, "satmixed": 2, "freeze": 3, "ice": 4, "snow": 5, "graupel": 6, "hail": 7,
            "settle": 8}[which]
    r = lib().orc_cell(code, fp(v), exner, p, rho, dt, aux)
    return r, {n: v[k] for k, n in enumerate(names)}
