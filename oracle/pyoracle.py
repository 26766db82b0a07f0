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
CHARGES = ("chargeIce", "chargeGraupel", "chargeRain", "chargeAir")
RAIN_NUMBER = "rainNumber"   # field id 17: raindrops per kg (two-moment rain)
ICE2M = ("graupelNumber", "graupelVolume", "hailNumber", "hailVolume")   # field ids 18-21 (two-moment graupel and hail)
EXTRA = {"precipitation": 100, "hailGround": 101, "hailSize": 102, "fallSpeed": 103, "snowFall": 104,
         "graupelFall": 105, "hailFall": 106, "condensate": 107, "chargeFallIce": 108, "chargeFallGraupel": 109,
         "fieldZ": 110, "rainFallNumber": 111, "graupelFallNumber": 112, "hailFallNumber": 113}

_d = C.POINTER(C.c_double)
_f = C.POINTER(C.c_float)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (plain g++/OpenMP)."""
    sources = [os.path.join(HERE, n) for n in ("oracle.cpp", "oracle_core.h", "oracle_solvers.h", "oracle_model.h", "oracle_diag.h",
                                               "oracle_elec.h", "oracle_rain2m.h", "oracle_ice2m.h", "oracle_terrain.h",
                                               os.path.join("..", "meteolab_gb300", "csrc", "sg_takahashi.h"))]
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
            L.orc_microphysics_2m.restype = C.c_double
            L.orc_microphysics_2m.argtypes = [_f, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_int)]
            L.orc_microphysics64.restype = C.c_double
            L.orc_microphysics64.argtypes = [_d, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
            L.orc_fft.argtypes = [C.c_int, _d, _d, C.c_int]
            L.orc_hdft.argtypes = [C.c_int, C.c_int, C.c_int, _d, _d, _d, _d]
            grid_args = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, _d, _d, _d]
            L.orc_pressure_project.argtypes = grid_args + [_d, _f, _f, _f, C.c_double, _d, _d, _d]
            L.orc_transport.argtypes = grid_args + [_d, _f, _f, _f, _f, C.c_double, C.c_int, C.c_int, _d, _d, _d, _d]
            L.orc_turbulence.argtypes = grid_args + [_d, _f, _f, _f, _f, _d, C.c_double, C.c_double, _f, _f, _d, C.c_int,
                                                     C.c_int, C.c_int, C.c_int, _d, _d, _d, _d, _f, _d, C.c_double, C.c_int]
            L.orc_set_lightning.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int]
            L.orc_charge_state.argtypes = [C.c_void_p, _d]
            L.orc_set_rain2m.argtypes = [C.c_void_p, C.c_int, C.c_int]
            for name, nargs in (("orc_r2m_bounded", 3), ("orc_r2m_mean_volume", 2), ("orc_r2m_dn", 1)):
                getattr(L, name).restype = C.c_double
                getattr(L, name).argtypes = [C.c_double] * nargs
            L.orc_r2m_fall.argtypes = [C.c_double] * 3 + [_d]
            L.orc_r2m_limits.restype = C.c_double
            L.orc_r2m_limits.argtypes = [C.c_int]
            L.orc_r2m_processes.restype = C.c_double
            L.orc_r2m_processes.argtypes = [_f] + [C.c_double] * 4 + [C.c_int, C.c_int]
            L.orc_r2m_number_change.argtypes = [_f, C.c_double, C.c_double, C.c_double]
            L.orc_set_ice2m.argtypes = [C.c_void_p, C.c_int]
            for name, args in (("orc_i2m_gamma", [C.c_double]), ("orc_i2m_upper_gamma", [C.c_int, C.c_double]),
                               ("orc_i2m_density", [C.c_int, C.c_double, C.c_double]),
                               ("orc_i2m_bounded", [C.c_int] + [C.c_double] * 3),
                               ("orc_i2m_moment_speed", [C.c_int] + [C.c_double] * 4 + [C.c_int]),
                               ("orc_i2m_largest", [C.c_int] + [C.c_double] * 4),
                               ("orc_i2m_reflectivity_factor", [C.c_int])):
                getattr(L, name).restype = C.c_double
                getattr(L, name).argtypes = args
            L.orc_i2m_fall_law.argtypes = [C.c_double, _d]
            L.orc_i2m_rimer_moments.restype = C.c_int
            L.orc_i2m_rimer_moments.argtypes = [C.c_int] + [C.c_double] * 4 + [_d]
            L.orc_i2m_sweep_coefficients.argtypes = [C.c_int, C.c_int, C.c_int, _d]
            L.orc_i2m_processes.argtypes = [_f] + [C.c_double] * 4 + [_d]
            _i = C.POINTER(C.c_int)
            L.orc_charging_rate_2m.restype = C.c_double
            L.orc_charging_rate_2m.argtypes = [C.c_double] * 8 + [C.c_int, C.c_int, C.c_double, _d, _i]
            L.orc_flash.argtypes = [C.c_void_p, C.c_int, _d, _i, _i, _i, _d, C.c_int]
            L.orc_lightning_create.restype = C.c_void_p
            L.orc_lightning_create.argtypes = grid_args + [_d, C.c_int]
            L.orc_lightning_destroy.argtypes = [C.c_void_p]
            L.orc_lightning_set_corona.argtypes = [C.c_void_p, C.c_int]
            L.orc_lightning_cloud.argtypes = [C.c_void_p, C.POINTER(_f), C.c_int]
            L.orc_lightning_solve.argtypes = [C.c_void_p, C.POINTER(_f)]
            L.orc_lightning_strongest.argtypes = [C.c_void_p, C.c_int, _d]
            L.orc_lightning_discharge.argtypes = [C.c_void_p, C.POINTER(_f), C.c_double, C.c_int]
            L.orc_lightning_flash.argtypes = [C.c_void_p, C.c_int, _d, _i, _i, _i, _d, C.c_int]
            L.orc_lightning_conduct.restype = C.c_double
            L.orc_lightning_conduct.argtypes = [C.c_void_p, _f, C.c_double]
            L.orc_lightning_fields.argtypes = [C.c_void_p, _d, _d, _d]
            L.orc_flash_limit.argtypes = [C.c_double]
            for name, nargs in (("orc_critical_rar", 1), ("orc_crystal_number", 3), ("orc_crystal_diameter", 3), ("orc_takahashi", 2)):
                getattr(L, name).restype = C.c_double
                getattr(L, name).argtypes = [C.c_double] * nargs
            L.orc_collision_charge.restype = C.c_double
            L.orc_collision_charge.argtypes = [C.c_double] * 4 + [C.c_int]
            L.orc_charging_rate.restype = C.c_double
            L.orc_charging_rate.argtypes = [C.c_double] * 8 + [C.c_int, C.c_int, C.c_double, C.c_int]
            L.orc_inductive_rate.restype = C.c_double
            L.orc_inductive_rate.argtypes = [C.c_double] * 7 + [C.c_int, C.c_int]
            L.orc_transfer_charge.argtypes = [_d, _d, _d]
            _u8 = C.POINTER(C.c_uint8)
            L.orc_terrain_heights.argtypes = grid_args + [C.c_int] + [C.c_double] * 6 + [_f]
            L.orc_terrain_geometry.argtypes = grid_args + [_f, _u8, _i, _d, _d, _d, _f]
            L.orc_masked_faces.argtypes = grid_args + [_d, _f, C.c_double, C.c_int, _f, _f, _f, _d, _d, _d, _d, _d]
            L.orc_masked_project.argtypes = grid_args + [_d, _f, C.c_double, C.c_int, _f, _f, _f, C.c_double, _d, _d, _d, _d, _u8]
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
                     sw.vertical_dz, sw.durran_klemp, sw.pressure_in_stages, getattr(sw, "ice", 1), 0.0, 0.0, 1, slabs],
                    dtype=np.float64)


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
        sw_ = spec.switches
        if getattr(sw_, "rain_moments", 1) == 2:
            L.orc_set_rain2m(self.h, 2, int(getattr(sw_, "rain_breakup", 0)))
        if getattr(sw_, "ice_moments", 1) == 2:
            L.orc_set_ice2m(self.h, 2)
        if getattr(sw_, "lightning", False):
            L.orc_set_lightning(self.h, 1, 1 if getattr(sw_, "corona", True) else 0, int(getattr(sw_, "lightning_seed", 43)))
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
        if name in CARRIED:
            return CARRIED.index(name)
        if name in CHARGES:
            return len(CARRIED) + CHARGES.index(name)
        if name == RAIN_NUMBER:
            return len(CARRIED) + len(CHARGES)
        if name in ICE2M:
            return len(CARRIED) + len(CHARGES) + 1 + ICE2M.index(name)
        return EXTRA[name]

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


CHARGE_STATE = ("chargeGround", "separated", "ic", "cgNegative", "cgPositive", "precipitation", "conduction", "flashesIC",
                "flashesCG", "totalCharge", "lastFlashes")


def _flash_record(read, k: int, cap: int = 3000):
    out, strokes = np.empty(9), np.zeros(8)
    nodes, parent, polarity = (np.empty(cap, np.int32) for _ in range(3))
    ip = C.POINTER(C.c_int)
    if read(k, dp(out), nodes.ctypes.data_as(ip), parent.ctypes.data_as(ip), polarity.ctypes.data_as(ip), dp(strokes), cap):
        return None
    m = int(out[7])
    return dict(time=out[0], kind="CG" if out[1] else "IC", start=int(out[2]), ground=int(out[3]), potential=out[4],
                charge=out[5], moment=out[6], nodes=nodes[:m].copy(), parent=parent[:m].copy(),
                polarity=polarity[:m].copy(), strokes=strokes[:int(out[8])].copy())


def _charge_state(self):
    out = np.empty(len(CHARGE_STATE))
    lib().orc_charge_state(self.h, dp(out))
    return dict(zip(CHARGE_STATE, out))


def _last_flashes(self):
    n = int(self.charge_state()["lastFlashes"])
    return [_flash_record(lambda *a: lib().orc_flash(self.h, *a), k) for k in range(n)]


OracleModel.charge_state = _charge_state
OracleModel.last_flashes = _last_flashes


def _float_ptrs(arrays):
    ptrs = (_f * len(arrays))(*[a.ctypes.data_as(_f) for a in arrays])
    return ptrs


class OracleLightning:
    """Lightning (src/core/lightning.ts:135-420) on a grid with the air density of each level: FP32 carriers (C/kg)
    changed in place, as the reference's Float32Arrays."""

    def __init__(self, grid, air, seed: int = 1):
        args, keep = grid_args(grid)
        self.grid, self.air = grid, f64(air)
        self.h = lib().orc_lightning_create(*args, dp(self.air), seed)
        self._keep = keep

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().orc_lightning_destroy(h)
            self.h = None

    @staticmethod
    def _check(carriers):
        for c in carriers:
            assert c.dtype == np.float32 and c.flags.c_contiguous

    def set_corona(self, on: bool):
        lib().orc_lightning_set_corona(self.h, 1 if on else 0)

    def cloud(self, fields):
        self._check(fields)
        lib().orc_lightning_cloud(self.h, _float_ptrs(fields), len(fields))

    def solve(self, carriers):
        self._check(carriers)
        lib().orc_lightning_solve(self.h, _float_ptrs(carriers))

    def strongest(self, stamp: int = -1):
        r = C.c_double()
        best = lib().orc_lightning_strongest(self.h, stamp, C.byref(r))
        return best, r.value

    def discharge(self, carriers, time: float, limit: int = 10):
        self._check(carriers)
        n = lib().orc_lightning_discharge(self.h, _float_ptrs(carriers), time, limit)
        return [_flash_record(lambda *a: lib().orc_lightning_flash(self.h, *a), k) for k in range(n)]

    def conduct(self, ions, dt: float) -> float:
        self._check([ions])
        return lib().orc_lightning_conduct(self.h, ions.ctypes.data_as(_f), dt)

    def fields(self):
        n = self.grid.nx * self.grid.ny * self.grid.nz
        phi, rho, st = np.empty(n), np.empty(n), np.empty(2)
        lib().orc_lightning_fields(self.h, dp(phi), dp(rho), dp(st))
        return phi, rho, dict(fromGround=st[0], conducted=st[1])


BREAKUP = {"none": 0, "nssl": 1, "morrison": 2}


def r2m_bounded(q, n, rho):
    return lib().orc_r2m_bounded(q, n, rho)


def r2m_mean_volume(q, n):
    return lib().orc_r2m_mean_volume(q, n)


def r2m_dn(xv):
    return lib().orc_r2m_dn(xv)


def r2m_limits():
    """(XV_MIN, XV_MAX, RAIN_MIN) of rain2m.ts."""
    return tuple(lib().orc_r2m_limits(k) for k in range(3))


def r2m_fall(q, n, rho):
    """(mass-weighted, number-weighted, reflectivity-weighted) fall speeds."""
    out = np.empty(3)
    lib().orc_r2m_fall(q, n, rho, dp(out))
    return tuple(out)


def r2m_processes(cell: np.ndarray, tk, p, rho, dt, breakup="none", evaporate=True):
    """rain2mProcesses on a float32 cell [q, cloud, rain, number] in place; returns the evaporated rain."""
    assert cell.dtype == np.float32 and cell.size == 4
    return lib().orc_r2m_processes(fp(cell), tk, p, rho, dt, BREAKUP[breakup], 1 if evaporate else 0)


def r2m_number_change(cell: np.ndarray, before, rho, mean_mass):
    """rainNumberChange on a float32 cell [rain, number] in place."""
    lib().orc_r2m_number_change(fp(cell), before, rho, mean_mass)


def flash_limit(dt: float) -> int:
    return lib().orc_flash_limit(dt)


def critical_rar(tc):
    return lib().orc_critical_rar(tc)


def collision_charge(tc, rar, d, v, signed=False):
    return lib().orc_collision_charge(tc, rar, d, v, 1 if signed else 0)


def crystal_number(tc, qi=0.0, rho=1.0):
    return lib().orc_crystal_number(tc, qi, rho)


def crystal_diameter(qi, rho, tc):
    return lib().orc_crystal_diameter(qi, rho, tc)


def takahashi(tc, lwc):
    return lib().orc_takahashi(tc, lwc)


def charging_rate(tc, rho, cloud, ice, snow, graupel, hail, snow_fall, wet_graupel=False, wet_hail=False, crystals=None,
                  scheme="tak"):
    return lib().orc_charging_rate(tc, rho, cloud, ice, snow, graupel, hail, snow_fall, int(wet_graupel), int(wet_hail),
                                   -1.0 if crystals is None else crystals, 1 if scheme == "tak" else 0)


def inductive_rate(tc, rho, cloud, graupel, hail, ez, rimer_charge, wet_graupel=False, wet_hail=False):
    return lib().orc_inductive_rate(tc, rho, cloud, graupel, hail, ez, rimer_charge, int(wet_graupel), int(wet_hail))


def transfer_charge(charge, before, after):
    c, b, a = f64(charge).copy(), f64(before), f64(after)
    lib().orc_transfer_charge(dp(c), dp(b), dp(a))
    return c


# ---------------------------------------------------------------- two-moment graupel and hail (src/core/ice2m.ts)
ICE_CLASS = {"graupel": 0, "hail": 1}
I2M_ORDER = ("theta", "q", "cloud", "ice", "iceNumber", "snow", "rain", "rainNumber", "graupel", "graupelNumber",
             "graupelVolume", "hail", "hailNumber", "hailVolume")


def i2m_gamma(x):
    return lib().orc_i2m_gamma(x)


def i2m_upper_gamma(n, x):
    return lib().orc_i2m_upper_gamma(n, x)


def i2m_fall_law(rho_x):
    out = np.zeros(2)
    lib().orc_i2m_fall_law(rho_x, dp(out))
    return float(out[0]), float(out[1])


def i2m_density(c, q, vol):
    return lib().orc_i2m_density(ICE_CLASS[c], q, vol)


def i2m_bounded(c, q, n, vol):
    return lib().orc_i2m_bounded(ICE_CLASS[c], q, n, vol)


def i2m_moment_speed(c, q, n, vol, rho, k):
    return lib().orc_i2m_moment_speed(ICE_CLASS[c], q, n, vol, rho, k)


def i2m_largest(c, q, n, vol, rho):
    return lib().orc_i2m_largest(ICE_CLASS[c], q, n, vol, rho)


def i2m_reflectivity_factor(c):
    return lib().orc_i2m_reflectivity_factor(ICE_CLASS[c])


def i2m_rimer_moments(c, q, n, vol, rho):
    """(n, d1, d2, fall, d2v) per m3, or None without the class."""
    out = np.zeros(5)
    return tuple(float(x) for x in out) if lib().orc_i2m_rimer_moments(ICE_CLASS[c], q, n, vol, rho, dp(out)) else None


def i2m_sweep_coefficients(c, y, k):
    """delbk(x, 0), delabk(x, y, k), delbk(y, k) for class c and y "droplets" or "exponential"."""
    out = np.zeros(3)
    lib().orc_i2m_sweep_coefficients(ICE_CLASS[c], 0 if y == "droplets" else 1, k, dp(out))
    return tuple(float(x) for x in out)


def i2m_node(**values) -> np.ndarray:
    """An FP32 cell vector in ice2mProcesses' field order, zero where not given."""
    return np.array([values.get(k, 0.0) for k in I2M_ORDER], np.float32)


def i2m_processes(cell: np.ndarray, exner, p, rho, dt):
    """ice2mProcesses on one node's cells (in place); returns (cooling, wetG, wetH)."""
    assert cell.dtype == np.float32 and cell.size == 14
    out = np.zeros(3)
    lib().orc_i2m_processes(fp(cell), exner, p, rho, dt, dp(out))
    return float(out[0]), bool(out[1]), bool(out[2])


def charging_rate_2m(tc, rho, cloud, ice, snow, graupel, hail, snow_fall, wet_g=False, wet_h=False, crystals=-1.0, moments=(None, None)):
    """chargingRate (Takahashi) with the two-moment moments of graupel and hail where given."""
    m = np.zeros(10)
    has = (C.c_int * 2)(*(0 if x is None else 1 for x in moments))
    for j, x in enumerate(moments):
        if x is not None:
            m[5 * j:5 * j + 5] = x
    return lib().orc_charging_rate_2m(tc, rho, cloud, ice, snow, graupel, hail, snow_fall, int(wet_g), int(wet_h), crystals, dp(m), has)


TERRAIN_KINDS = {"hill": 0, "ridge": 1, "plateau": 2, "schar": 3}


def terrain_heights(grid, kind: str, height: float, width: float, x=None, y=None, heading=None, wavelength=None) -> np.ndarray:
    """terrainHeights (src/core/terrain.ts:37-63): the ground height of every column, m, float32 [ny*nx]."""
    L = lib()
    args, keep = grid_args(grid)
    out = np.zeros(grid.nx * grid.ny, np.float32)
    opt = [float("nan") if a is None else float(a) for a in (x, y, heading, wavelength)]
    L.orc_terrain_heights(*args, TERRAIN_KINDS[kind], height, width, *opt, fp(out))
    return out


def terrain_geometry(grid, ground: np.ndarray) -> Dict[str, np.ndarray]:
    """solidMask, groundLevels, nodeHeights, faceApertures and slopeArea (src/core/terrain.ts:80-150) of ground heights."""
    L = lib()
    args, keep = grid_args(grid)
    g = np.ascontiguousarray(ground, dtype=np.float32)
    n, layer = grid.nx * grid.ny * grid.nz, grid.nx * grid.ny
    out = {"solid": np.zeros(n, np.uint8), "levels": np.zeros(layer, np.int32), "heights": np.zeros(n), "ax": np.zeros(n),
           "ay": np.zeros(n), "slope": np.zeros(layer, np.float32)}
    L.orc_terrain_geometry(*args, fp(g), out["solid"].ctypes.data_as(C.POINTER(C.c_uint8)), out["levels"].ctypes.data_as(C.POINTER(C.c_int)),
                           dp(out["heights"]), dp(out["ax"]), dp(out["ay"]), fp(out["slope"]))
    return out


def masked_project(grid, rho, ground, u, v, w, dt, pressure=None, tolerance=1e-6, max_iterations=200):
    """MaskedProjection (src/core/terrain.ts:168-363) as the reference's test drives it (terrain.test.ts:23-45): mask,
    the cut cells' divergence before, project in place, the divergence after. Returns (u, v, w, pressure, before, after,
    iterations, residual, dropped)."""
    L = lib()
    args, keep = grid_args(grid)
    cells = grid.nx * grid.ny * (grid.nz - 1)
    uu, vv, ww = (np.array(a, dtype=np.float32, copy=True) for a in (u, v, w))
    p = np.zeros(cells) if pressure is None else np.array(pressure, dtype=np.float64, copy=True)
    before, after, stats, dropped = np.zeros(cells), np.zeros(cells), np.zeros(2), np.zeros(cells, np.uint8)
    r, g = f64(rho), np.ascontiguousarray(ground, dtype=np.float32)
    L.orc_masked_project(*args, dp(r), fp(g), tolerance, max_iterations, fp(uu), fp(vv), fp(ww), dt, dp(p), dp(before), dp(after),
                         dp(stats), dropped.ctypes.data_as(C.POINTER(C.c_uint8)))
    return uu, vv, ww, p, before, after, int(stats[0]), float(stats[1]), dropped


def masked_faces(grid, rho, ground, u, v, w, tolerance=1e-10, max_iterations=400):
    """FluxTransport.setVelocityMasked (src/core/advection.ts:115-153) with the model's terrain set-up (model.ts:366-377):
    the projected face mass fluxes mx, my, mz, their divergence over the node heights, iterations and residual."""
    L = lib()
    args, keep = grid_args(grid)
    n = grid.nx * grid.ny * grid.nz
    mx, my, mz, div, stats = np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(n), np.zeros(2)
    uu, vv, ww = (np.ascontiguousarray(a, dtype=np.float32) for a in (u, v, w))
    L.orc_masked_faces(*args, dp(f64(rho)), fp(np.ascontiguousarray(ground, dtype=np.float32)), tolerance, max_iterations, fp(uu), fp(vv), fp(ww),
                       dp(mx), dp(my), dp(mz), dp(div), dp(stats))
    return mx, my, mz, div, int(stats[0]), float(stats[1])
