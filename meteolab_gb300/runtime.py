"""Python host side over the C ABI of libstormgpu.so (include/stormgpu.h).

Mirrors the reference's interface for the step: ``AtmosphereModel(config, grid, profile)`` with ``step(dt)`` and the
model's fields as arrays (src/core/model.ts:183-210, :329, :873), here backed by a device-resident run. There is no
CPU fallback: without the built library or a CUDA device every call raises ``StormGpuError``.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import threading
from typing import Dict, Iterable, List, Optional, Sequence

import numpy as np

from .scenarios import CARRIED, CHARGES, ICE2M, RunSpec

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libstormgpu.so")

STATUS = {0: "ok", 1: "invalid", 2: "budget", 3: "device", 4: "timeout", 5: "non-finite", 6: "not found", 7: "unsupported"}


class StormGpuError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"stormgpu {STATUS.get(code, code)}: {message}")
        self.code = code


class SgGrid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("reserved", C.c_int32),
                ("dx", C.c_double), ("dy", C.c_double), ("height", C.c_double),
                ("zs", C.POINTER(C.c_double)), ("dzs", C.POINTER(C.c_double)), ("hz", C.POINTER(C.c_double))]


class SgTerrain(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("height", C.c_double), ("width", C.c_double), ("x", C.c_double),
                ("y", C.c_double), ("heading", C.c_double), ("wavelength", C.c_double)]


class SgBase(C.Structure):
    _fields_ = [(k, C.POINTER(C.c_double)) for k in ("p", "exner", "theta", "q", "u", "v", "rho")]


class SgSwitches(C.Structure):
    _fields_ = [("dt", C.c_double), ("coriolis", C.c_double), ("wind_relaxation", C.c_double), ("sponge_rate", C.c_double),
                ("sponge_start", C.c_double), ("cs", C.c_double), ("drag_cd", C.c_double), ("frame_u", C.c_double),
                ("frame_v", C.c_double)] + [(k, C.c_int32) for k in ("loading", "evaporation", "rain_formation",
                                                                         "anisotropic", "vertical_dz", "durran_klemp",
                                                                         "pressure_in_stages", "ice", "refine_projection",
                                                                         "rotation", "lightning", "corona", "lightning_seed",
                                                                         "rain_moments", "rain_breakup", "ice_moments")]


class SgChargeState(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("ground", "separated", "ic", "cg_negative", "cg_positive", "precipitation", "conduction")] + \
               [("flashes_ic", C.c_int64), ("flashes_cg", C.c_int64), ("last_flashes", C.c_int32), ("electrified", C.c_int32)]


class SgFlash(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("time", "potential", "charge", "moment")] + [("stroke_charge", C.c_double * 4)] + \
               [(k, C.c_int32) for k in ("cg", "start", "ground", "nodes", "strokes", "reserved")]


class SgStateInfo(C.Structure):
    _fields_ = [("version", C.c_int32), ("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("nfields", C.c_int32),
                ("reserved", C.c_int32), ("time", C.c_double), ("persisted", C.c_double), ("data_offset", C.c_uint64)]


class SgRotation(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("uh", "x", "y", "anticyclonic", "persisted", "uh01", "uh03", "low", "coreZeta", "coreUH",
                                          "coreAnti", "time")]


class SgDiagnostics(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("updraft", "downdraft", "rainRate", "rainTotal", "cloudTop", "thermalTop", "maxCloud",
                                          "coldMax", "cores", "outflow", "outflowLow", "gust", "hail", "clipped")]


class SgCounters(C.Structure):
    _fields_ = [("steps", C.c_int64), ("clipped", C.c_int64), ("negative_filled", C.c_double),
                ("water_condensed", C.c_double), ("water_evaporated", C.c_double), ("water_rain_evaporated", C.c_double),
                ("water_surface", C.c_double), ("failed", C.c_int32), ("reserved", C.c_int32)]


_lib = None
_lock = threading.Lock()
# field ids of the C ABI (charges: electrified runs; drop number: two-moment rain; graupel and hail numbers and volumes:
# two-moment ice)
ALL_FIELDS = tuple(CARRIED) + tuple(CHARGES) + ("rainNumber",) + tuple(ICE2M)
_FP = C.POINTER(C.c_float)


def load():
    """Load the in-tree libstormgpu.so (build it first with meteolab_gb300.build.build())."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise StormGpuError(3, f"{LIB_PATH} is not built; run meteolab_gb300.build.build()")
            L = C.CDLL(LIB_PATH)
            vp, i32, u64, i64 = C.c_void_p, C.c_int, C.c_uint64, C.c_int64
            L.sg_context_create.argtypes = [i32, u64, C.POINTER(vp)]
            L.sg_context_destroy.argtypes = [vp]
            L.sg_last_error.restype = C.c_char_p
            L.sg_last_error.argtypes = [vp]
            L.sg_run_bytes.restype = u64
            L.sg_run_bytes.argtypes = [C.POINTER(SgGrid)]
            L.sg_run_create.argtypes = [vp, C.POINTER(SgGrid), C.POINTER(SgBase), C.POINTER(SgSwitches), C.POINTER(_FP), C.POINTER(C.c_int32)]
            L.sg_run_write_fields.argtypes = [vp, C.c_int32, C.c_uint32, C.POINTER(_FP)]
            L.sg_run_read_fields.argtypes = [vp, C.c_int32, C.c_uint32, C.POINTER(_FP)]
            L.sg_run_read_columns.argtypes = [vp, C.c_int32, _FP, _FP, _FP]
            L.sg_run_read_pressure.argtypes = [vp, C.c_int32, C.POINTER(C.c_double)]
            L.sg_run_status.argtypes = [vp, C.c_int32, C.POINTER(SgCounters)]
            L.sg_run_retire.argtypes = [vp, C.c_int32]
            L.sg_run_step.argtypes = [vp, C.c_int32, i32]
            L.sg_batch_step.argtypes = [vp, C.POINTER(C.c_int32), i32, i32]
            L.sg_batch_step_async.argtypes = [vp, C.POINTER(C.c_int32), i32, i32]
            L.sg_synchronize.argtypes = [vp]
            L.sg_profile_kernels.argtypes = [vp, C.POINTER(C.c_int32), i32, i32, C.POINTER(C.c_char_p), C.POINTER(C.c_double),
                                             C.POINTER(C.c_int64), i32]
            L.sg_run_divergence.argtypes = [vp, C.c_int32, C.POINTER(C.c_double)]
            L.sg_time_steps.argtypes = [vp, C.POINTER(C.c_int32), i32, i32, i32, C.POINTER(C.c_double)]
            L.sg_debug_step_part.argtypes = [vp, C.c_int32, i32]
            L.sg_debug_read_set.argtypes = [vp, C.c_int32, i32, i32, _FP]
            L.sg_debug_read_faces.argtypes = [vp, C.c_int32, _FP]
            L.sg_batch_write_fields.argtypes = [vp, C.POINTER(C.c_int32), i32, C.c_uint32, C.POINTER(_FP)]
            L.sg_batch_read_fields.argtypes = [vp, C.POINTER(C.c_int32), i32, C.c_uint32, C.POINTER(_FP)]
            L.sg_batch_write_packed.argtypes = [vp, C.POINTER(C.c_int32), i32, C.c_uint32, _FP]
            L.sg_electric_create.argtypes = [vp, C.POINTER(SgGrid), C.POINTER(vp)]
            L.sg_electric_solve.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.sg_electric_destroy.argtypes = [vp]
            _U8 = C.POINTER(C.c_uint8)
            L.sg_terrain_heights.argtypes = [C.POINTER(SgGrid), C.POINTER(SgTerrain), _FP]
            L.sg_terrain_geometry.argtypes = [C.POINTER(SgGrid), _FP, _U8, C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                              C.POINTER(C.c_double), C.POINTER(C.c_double), _FP]
            L.sg_masked_create.argtypes = [vp, C.POINTER(SgGrid), C.POINTER(C.c_double), _FP, C.c_double, i32, C.POINTER(vp)]
            L.sg_masked_project.argtypes = [vp, _FP, _FP, _FP, C.c_double, C.POINTER(C.c_double)]
            L.sg_masked_mask.argtypes = [vp, _FP, _FP, _FP]
            L.sg_masked_divergence.argtypes = [vp, _FP, _FP, _FP, C.POINTER(C.c_double)]
            L.sg_masked_stats.argtypes = [vp, C.POINTER(C.c_int32), C.POINTER(C.c_double)]
            L.sg_masked_dropped.argtypes = [vp, _U8]
            L.sg_masked_destroy.argtypes = [vp]
            _D = C.POINTER(C.c_double)
            L.sg_faces_create.argtypes = [vp, C.POINTER(SgGrid), _D, _FP, C.c_double, i32, C.POINTER(vp)]
            L.sg_faces_set_velocity.argtypes = [vp, _FP, _FP, _FP, _D, _D, _D, _D]
            L.sg_faces_stats.argtypes = [vp, C.POINTER(C.c_int32), _D]
            L.sg_faces_destroy.argtypes = [vp]
            L.sg_batch_read_packed.argtypes = [vp, C.POINTER(C.c_int32), i32, C.c_uint32, _FP]
            L.sg_batch_step_io.argtypes = [vp, C.POINTER(C.c_int32), i32, C.c_uint32, _FP, i32, i32]
            L.sg_batch_step_round_trips.argtypes = [vp, C.POINTER(C.c_int32), i32, C.c_uint32, _FP, i32, i32]
            L.sg_set_transport_shape.argtypes = [vp, i32, i32, i32]
            L.sg_divergence_max_static.argtypes = [i32, vp, vp, vp, i32, i32, i32, C.c_double, C.c_double, C.POINTER(C.c_double),
                                                   C.POINTER(C.c_double), vp, C.POINTER(C.c_double), C.c_char_p, C.c_size_t]
            L.sg_batch_transport_shape.argtypes = [vp, C.POINTER(C.c_int32), i32, C.POINTER(C.c_int)]
            L.sg_batch_transport_copies.argtypes = [vp, C.POINTER(C.c_int32), i32, C.POINTER(C.c_int)]
            L.sg_server_create.argtypes = [vp, i32, C.POINTER(vp)]
            L.sg_server_destroy.argtypes = [vp]
            L.sg_server_submit.argtypes = [vp, C.POINTER(SgGrid), C.POINTER(SgBase), C.POINTER(SgSwitches), C.POINTER(_FP), i64, i64]
            L.sg_server_iterate.argtypes = [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int), i32, C.POINTER(C.c_int), C.POINTER(C.c_int)]
            L.sg_server_collect.argtypes = [vp, i64, C.c_uint32, C.POINTER(_FP), _FP]
            L.sg_server_set_quantum.argtypes = [vp, i32]
            L.sg_server_last_steps.argtypes = [vp]
            L.sg_run_write_columns.argtypes = [vp, C.c_int32, _FP, _FP, _FP]
            L.sg_run_shape.argtypes = [vp, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
            L.sg_state_parse.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(SgStateInfo), C.c_char_p, C.c_size_t]
            L.sg_run_save_state.argtypes = [vp, C.c_int32, C.c_char_p, C.c_double, C.c_double, C.c_char_p, C.c_size_t,
                                            C.POINTER(C.c_size_t)]
            L.sg_run_load_state.argtypes = [vp, C.c_int32, C.c_char_p, C.c_size_t, C.POINTER(SgStateInfo)]
            L.sg_run_rotation.argtypes = [vp, C.c_int32, C.POINTER(SgRotation), _FP]
            L.sg_run_refresh_rotation.argtypes = [vp, C.c_int32]
            L.sg_run_read_swaths.argtypes = [vp, C.c_int32, _FP, _FP]
            L.sg_run_reset_swaths.argtypes = [vp, C.c_int32]
            L.sg_run_diagnostics.argtypes = [vp, C.c_int32, C.POINTER(SgDiagnostics)]
            L.sg_run_bytes_for.restype = u64
            L.sg_run_bytes_for.argtypes = [C.POINTER(SgGrid), C.POINTER(SgSwitches)]
            L.sg_run_charge.argtypes = [vp, C.c_int32, C.POINTER(SgChargeState)]
            L.sg_run_flashes.argtypes = [vp, C.c_int32, C.POINTER(SgFlash), i32, C.POINTER(C.c_int)]
            L.sg_run_flash_channel.argtypes = [vp, C.c_int32, i32, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32), i32]
            L.sg_run_discharge.argtypes = [vp, C.c_int32, C.c_double, C.c_double]
            L.sg_debug_lightning.argtypes = [vp, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int32),
                                             C.POINTER(C.c_double), C.POINTER(C.c_double)]
            _lib = L
    return _lib


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _switches(sw, g) -> "SgSwitches":
    """The POD sg_switches of a ``scenarios.Switches`` on grid g."""
    return SgSwitches(sw.dt, sw.coriolis, sw.wind_relaxation, sw.sponge_rate, sw.sponge_start, sw.cs, sw.drag_cd(g),
                      sw.frame_u, sw.frame_v, sw.loading, sw.evaporation, sw.rain_formation, sw.anisotropic,
                      sw.vertical_dz, sw.durran_klemp, sw.pressure_in_stages, getattr(sw, "ice", 1),
                      sw.refine_projection, sw.rotation, getattr(sw, "lightning", 0), getattr(sw, "corona", 1),
                      getattr(sw, "lightning_seed", 43), getattr(sw, "rain_moments", 1), getattr(sw, "rain_breakup", 0),
                      getattr(sw, "ice_moments", 1))


class _Packed:
    """The C structs of one run spec with the arrays they point to kept alive."""

    def __init__(self, spec: RunSpec):
        g, env, sw = spec.grid, spec.env, spec.switches
        self.keep = [_f64(g.zs), _f64(g.dzs), _f64(g.hz)] + [_f64(getattr(env, k)) for k in ("p", "exner", "theta", "q", "u", "v", "rho")]
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self.grid = SgGrid(g.nx, g.ny, g.nz, 0, g.dx, g.dy, g.height, dp(self.keep[0]), dp(self.keep[1]), dp(self.keep[2]))
        self.base = SgBase(*[dp(a) for a in self.keep[3:]])
        self.switches = _switches(sw, g)
        self.fields = [np.ascontiguousarray(spec.fields[k], dtype=np.float32).ravel() for k in CARRIED]
        self.ptrs = (_FP * len(CARRIED))(*[a.ctypes.data_as(_FP) for a in self.fields])


def run_bytes(grid, switches=None) -> int:
    """Bytes of HBM one run of this grid takes in a context (sg_run_bytes; with `switches`, sg_run_bytes_for: an
    electrified or two-moment run's extra fields and buffers): what admission by budget counts."""
    zs, dzs, hz = _f64(grid.zs), _f64(grid.dzs), _f64(grid.hz)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    g = SgGrid(grid.nx, grid.ny, grid.nz, 0, grid.dx, grid.dy, grid.height, dp(zs), dp(dzs), dp(hz))
    if switches is None:
        return int(load().sg_run_bytes(C.byref(g)))
    sw = _switches(switches, grid)
    return int(load().sg_run_bytes_for(C.byref(g), C.byref(sw)))


class Context:
    """One device context (one CUDA stream, an HBM budget, the runs it owns)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        L = load()
        h = C.c_void_p()
        rc = L.sg_context_create(device, hbm_budget, C.byref(h))
        if rc:
            raise StormGpuError(rc, "sg_context_create failed (is a CUDA device visible?)")
        self.h = h

    def check(self, rc: int, what: str = ""):
        if rc:
            raise StormGpuError(rc, f"{what}: {load().sg_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            load().sg_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def create(self, spec: RunSpec) -> "Run":
        return Run(self, spec)

    def batch_step(self, runs: Sequence["Run"], steps: int = 1, wait: bool = True):
        ids = (C.c_int32 * len(runs))(*[r.id for r in runs])
        fn = load().sg_batch_step if wait else load().sg_batch_step_async
        self.check(fn(self.h, ids, len(runs), steps), "batch step")
        for r in runs:
            r.time += steps * r.spec.switches.dt

    def time_steps(self, runs: Sequence["Run"], steps: int, graph: bool = True) -> float:
        """Device time (ms, CUDA events on the library's stream) of `steps` batch steps."""
        ids = (C.c_int32 * len(runs))(*[r.id for r in runs])
        ms = C.c_double()
        self.check(load().sg_time_steps(self.h, ids, len(runs), steps, 1 if graph else 0, C.byref(ms)), "time steps")
        for r in runs:
            r.time += steps * r.spec.switches.dt
        return ms.value

    def _batch_io(self, runs, bufs, names, write: bool):
        names = list(names)
        mask = 0
        for k in names:
            mask |= 1 << CARRIED.index(k)
        ptrs = (_FP * (len(runs) * len(CARRIED)))()
        keep = []
        for j, (r, b) in enumerate(zip(runs, bufs)):
            for k in names:
                a = b[k]
                if write:
                    a = np.ascontiguousarray(a, dtype=np.float32).ravel()
                    keep.append(a)
                elif a.dtype != np.float32 or not a.flags.c_contiguous or a.size != r.grid.n:
                    raise ValueError(f"output buffer for {k} must be a contiguous float32 array of {r.grid.n}")
                ptrs[j * len(CARRIED) + CARRIED.index(k)] = a.ctypes.data_as(_FP)
        ids = (C.c_int32 * len(runs))(*[r.id for r in runs])
        fn = load().sg_batch_write_fields if write else load().sg_batch_read_fields
        self.check(fn(self.h, ids, len(runs), mask, ptrs), "batch fields")

    def write_fields(self, runs: Sequence["Run"], fields: Sequence[Dict[str, np.ndarray]], names: Iterable[str] = CARRIED):
        """Write the fields of many runs in one call (one synchronisation)."""
        self._batch_io(runs, fields, names, True)

    def read_fields(self, runs: Sequence["Run"], out: Sequence[Dict[str, np.ndarray]], names: Iterable[str] = CARRIED):
        """Read the fields of many runs into the caller's float32 arrays in one call."""
        self._batch_io(runs, out, names, False)

    def _mask(self, names) -> int:
        m = 0
        for k in names:
            m |= 1 << CARRIED.index(k)
        return m

    def write_packed(self, runs: Sequence["Run"], packed: np.ndarray, names: Iterable[str] = CARRIED):
        """Write the fields of many runs from one buffer: run after run, the named fields in field order."""
        if packed.dtype != np.float32 or not packed.flags.c_contiguous:
            raise ValueError("packed buffer must be contiguous float32")
        ids = (C.c_int32 * len(runs))(*[r.id for r in runs])
        self.check(load().sg_batch_write_packed(self.h, ids, len(runs), self._mask(names), packed.ctypes.data_as(_FP)), "write packed")

    def read_packed(self, runs: Sequence["Run"], packed: np.ndarray, names: Iterable[str] = CARRIED):
        """Read the fields of many runs into one buffer (the layout of write_packed)."""
        if packed.dtype != np.float32 or not packed.flags.c_contiguous:
            raise ValueError("packed buffer must be contiguous float32")
        ids = (C.c_int32 * len(runs))(*[r.id for r in runs])
        self.check(load().sg_batch_read_packed(self.h, ids, len(runs), self._mask(names), packed.ctypes.data_as(_FP)), "read packed")

    def batch_step_io(self, runs: Sequence["Run"], packed: np.ndarray, steps: int = 1, groups: int = 4,
                      names: Iterable[str] = CARRIED):
        """Write the runs' fields from `packed` (the layout of write_packed), advance them `steps`, read them back into
        `packed`: the reference engine's per-step host round trip, with the runs cut into `groups` groups whose copies
        overlap the other groups' steps."""
        if packed.dtype != np.float32 or not packed.flags.c_contiguous:
            raise ValueError("packed buffer must be contiguous float32")
        ids = (C.c_int32 * len(runs))(*[r.id for r in runs])
        self.check(load().sg_batch_step_io(self.h, ids, len(runs), self._mask(names), packed.ctypes.data_as(_FP), steps, groups),
                   "batch step io")
        for r in runs:
            r.time += steps * r.spec.switches.dt

    def batch_round_trips(self, runs: Sequence["Run"], packed: np.ndarray, steps: int = 1, groups: int = 4,
                          names: Iterable[str] = CARRIED):
        """`steps` steps with the round trip every step (sg_batch_step_round_trips): each step writes the runs' fields
        from `packed`, advances one step and reads them back into it; the groups pipeline independently."""
        if packed.dtype != np.float32 or not packed.flags.c_contiguous:
            raise ValueError("packed buffer must be contiguous float32")
        ids = (C.c_int32 * len(runs))(*[r.id for r in runs])
        self.check(load().sg_batch_step_round_trips(self.h, ids, len(runs), self._mask(names), packed.ctypes.data_as(_FP), steps,
                                                    groups), "batch round trips")
        for r in runs:
            r.time += steps * r.spec.switches.dt

    def set_transport_shape(self, tile_x: int = 0, tile_y: int = 0, weno_group: int = 3):
        """Pin the transport tile (tile_x x tile_y columns, 1 or 3 WENO fields per item); tile_x = 0 returns to tuning."""
        self.check(load().sg_set_transport_shape(self.h, tile_x, tile_y, weno_group), "transport shape")

    def transport_shape(self, runs: Sequence["Run"]) -> tuple:
        """(tile_x, tile_y, weno_group, blocks per SM of the WENO kernel) the batch of `runs` is stepped with."""
        ids = (C.c_int32 * len(runs))(*[r.id for r in runs])
        out = (C.c_int * 4)()
        self.check(load().sg_batch_transport_shape(self.h, ids, len(runs), out), "transport shape")
        return tuple(out)

    def transport_bulk(self, runs: Sequence["Run"]) -> bool:
        """Whether the batch's transport tiles move their inputs by TMA bulk copies (sg_batch_transport_copies)."""
        ids = (C.c_int32 * len(runs))(*[r.id for r in runs])
        out = C.c_int()
        self.check(load().sg_batch_transport_copies(self.h, ids, len(runs), C.byref(out)), "transport copies")
        return bool(out.value)

    def synchronize(self):
        self.check(load().sg_synchronize(self.h), "synchronize")

    def profile(self, runs: Sequence["Run"], steps: int = 2) -> Dict[str, tuple]:
        """Mean device ms per launch of each kernel class over `steps` eager steps."""
        ids = (C.c_int32 * len(runs))(*[r.id for r in runs])
        cap = 32
        names = (C.c_char_p * cap)()
        ms = (C.c_double * cap)()
        launches = (C.c_int64 * cap)()
        n = load().sg_profile_kernels(self.h, ids, len(runs), steps, names, ms, launches, cap)
        if n < 0:
            self.check(-n, "profile")
        return {names[k].decode(): (ms[k], launches[k] // max(1, steps)) for k in range(n)}


class Run:
    """A device-resident run (the state of one model)."""

    def __init__(self, ctx: Context, spec: RunSpec):
        self.ctx, self.spec, self.grid = ctx, spec, spec.grid
        packed = _Packed(spec)
        rid = C.c_int32()
        ctx.check(load().sg_run_create(ctx.h, C.byref(packed.grid), C.byref(packed.base), C.byref(packed.switches), packed.ptrs,
                                       C.byref(rid)), "run create")
        self.id = rid.value
        self.time = 0.0
        self.live = True
        extra = {k: v for k, v in spec.fields.items() if k in CHARGES or k == "rainNumber" or k in ICE2M}
        if extra:
            self.write(extra)

    def retire(self):
        if self.live:
            self.ctx.check(load().sg_run_retire(self.ctx.h, self.id), "retire")
            self.live = False

    def step(self, steps: int = 1):
        self.ctx.check(load().sg_run_step(self.ctx.h, self.id, steps), "step")
        self.time += steps * self.spec.switches.dt

    def read(self, names: Iterable[str] = CARRIED, out: Optional[Dict[str, np.ndarray]] = None) -> Dict[str, np.ndarray]:
        names = list(names)
        out = out if out is not None else {k: np.empty(self.grid.n, np.float32) for k in names}
        mask = 0
        ptrs = (_FP * len(ALL_FIELDS))()
        for k in names:
            j = ALL_FIELDS.index(k)
            mask |= 1 << j
            ptrs[j] = out[k].ctypes.data_as(_FP)
        self.ctx.check(load().sg_run_read_fields(self.ctx.h, self.id, mask, ptrs), "read fields")
        return out

    def write(self, fields: Dict[str, np.ndarray]):
        mask = 0
        ptrs = (_FP * len(ALL_FIELDS))()
        keep = []
        for k, a in fields.items():
            j = ALL_FIELDS.index(k)
            a = np.ascontiguousarray(a, dtype=np.float32).ravel()
            keep.append(a)
            mask |= 1 << j
            ptrs[j] = a.ctypes.data_as(_FP)
        self.ctx.check(load().sg_run_write_fields(self.ctx.h, self.id, mask, ptrs), "write fields")

    def columns(self) -> Dict[str, np.ndarray]:
        layer = self.grid.layer
        out = {k: np.empty(layer, np.float32) for k in ("precipitation", "hailGround", "hailSize")}
        self.ctx.check(load().sg_run_read_columns(self.ctx.h, self.id, *[out[k].ctypes.data_as(_FP) for k in ("precipitation", "hailGround", "hailSize")]),
                       "read columns")
        return out

    def pressure(self) -> np.ndarray:
        out = np.empty(self.grid.nx * self.grid.ny * (self.grid.nz - 1))
        self.ctx.check(load().sg_run_read_pressure(self.ctx.h, self.id, out.ctypes.data_as(C.POINTER(C.c_double))), "read pressure")
        return out

    def status(self) -> dict:
        c = SgCounters()
        rc = load().sg_run_status(self.ctx.h, self.id, C.byref(c))
        if rc not in (0, 5):
            self.ctx.check(rc, "status")
        return {k: getattr(c, k) for k, _ in SgCounters._fields_ if k != "reserved"}

    def charge(self) -> dict:
        """The charge budget and flash counts (chargeGround, charge, flashCount, src/core/model.ts:218-241)."""
        c = SgChargeState()
        self.ctx.check(load().sg_run_charge(self.ctx.h, self.id, C.byref(c)), "charge")
        return {k: getattr(c, k) for k, _ in SgChargeState._fields_}

    def flashes(self, channels: bool = True) -> List[dict]:
        """The last step's flashes (Flash records, src/core/lightning.ts:69-106), with their channels."""
        count = C.c_int()
        self.ctx.check(load().sg_run_flashes(self.ctx.h, self.id, None, 0, C.byref(count)), "flashes")
        n = count.value
        recs = (SgFlash * max(1, n))()
        self.ctx.check(load().sg_run_flashes(self.ctx.h, self.id, recs, n, C.byref(count)), "flashes")
        out = []
        for k in range(n):
            f = recs[k]
            d = dict(time=f.time, kind="CG" if f.cg else "IC", start=f.start, ground=f.ground, potential=f.potential,
                     charge=f.charge, moment=f.moment, strokes=np.array(list(f.stroke_charge)[:f.strokes]))
            if channels:
                m = f.nodes
                nodes, parent, polarity = (np.empty(m, np.int32) for _ in range(3))
                ip = C.POINTER(C.c_int32)
                self.ctx.check(load().sg_run_flash_channel(self.ctx.h, self.id, k, nodes.ctypes.data_as(ip), parent.ctypes.data_as(ip),
                                                           polarity.ctypes.data_as(ip), m), "flash channel")
                d.update(nodes=nodes, parent=parent, polarity=polarity)
            out.append(d)
        return out

    LAST_FLASH = ("id", "start", "size", "nodes", "ground", "event", "left", "strokes", "grown", "potential", "sum",
                  "neutralized", "lowered", "stage", "charge", "flashId")

    def lightning_probe(self):
        """The discharge's first search on the charge as it stands: (phi, rho, strongest node, |E| / Einit there, the
        last flash's state record)."""
        n = self.grid.n
        phi, rho, best, ratio, last = np.empty(n), np.empty(n), C.c_int32(), C.c_double(), np.empty(16)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self.ctx.check(load().sg_debug_lightning(self.ctx.h, self.id, dp(phi), dp(rho), C.byref(best), C.byref(ratio), dp(last)),
                       "lightning probe")
        return phi, rho, best.value, ratio.value, dict(zip(self.LAST_FLASH, last))

    def discharge(self, time: float, dt: float):
        """AtmosphereModel.discharge on the run's charge as it stands (src/core/model.ts:1537-1552), at model time `time`."""
        self.ctx.check(load().sg_run_discharge(self.ctx.h, self.id, time, dt), "discharge")

    def debug_part(self, part: int):
        """Run one part of the step (1 beginStep, 2 dynamics, 3 physicsStep, 4 mixStep, 5 final projection)."""
        self.ctx.check(load().sg_debug_step_part(self.ctx.h, self.id, part), f"step part {part}")

    def debug_read_set(self, set_: int, name: str) -> np.ndarray:
        """A raw device buffer (theta of a set is its departure from the base profile)."""
        out = np.empty(self.grid.n, np.float32)
        self.ctx.check(load().sg_debug_read_set(self.ctx.h, self.id, set_, CARRIED.index(name), out.ctypes.data_as(_FP)), "read set")
        return out

    def debug_faces(self) -> np.ndarray:
        out = np.empty((self.grid.n, 4), np.float32)
        self.ctx.check(load().sg_debug_read_faces(self.ctx.h, self.id, out.ctypes.data_as(_FP)), "read faces")
        return out.T.copy()  # mx, my, mz, div

    def divergence(self) -> float:
        out = C.c_double()
        self.ctx.check(load().sg_run_divergence(self.ctx.h, self.id, C.byref(out)), "divergence")
        return out.value

    def write_columns(self, cols: Dict[str, np.ndarray]):
        keep = [np.ascontiguousarray(cols[k], dtype=np.float32) if k in cols else None for k in ("precipitation", "hailGround", "hailSize")]
        ptrs = [a.ctypes.data_as(_FP) if a is not None else None for a in keep]
        self.ctx.check(load().sg_run_write_columns(self.ctx.h, self.id, *ptrs), "write columns")

    def rotation(self, column: bool = False):
        """The rotation state after the last step (model.rotation, src/core/model.ts:263) and, with column=True, the
        2-5 km UH column (model.uhColumn)."""
        r = SgRotation()
        col = np.empty(self.grid.layer, np.float32) if column else None
        self.ctx.check(load().sg_run_rotation(self.ctx.h, self.id, C.byref(r), col.ctypes.data_as(_FP) if column else None), "rotation")
        out = {k: getattr(r, k) for k, _ in SgRotation._fields_}
        return (out, col) if column else out

    def refresh_rotation(self):
        """refreshRotation (src/core/model.ts:1607): the rotation from the fields as they are."""
        self.ctx.check(load().sg_run_refresh_rotation(self.ctx.h, self.id), "refresh rotation")

    def swaths(self) -> Dict[str, np.ndarray]:
        """The run's swaths (MemberResult.gustMax, uhMax, src/ensemble/member.ts:20-21)."""
        g, u = np.empty(self.grid.layer, np.float32), np.empty(self.grid.layer, np.float32)
        self.ctx.check(load().sg_run_read_swaths(self.ctx.h, self.id, g.ctypes.data_as(_FP), u.ctypes.data_as(_FP)), "swaths")
        return {"gustMax": g, "uhMax": u}

    def reset_swaths(self):
        self.ctx.check(load().sg_run_reset_swaths(self.ctx.h, self.id), "reset swaths")

    def diagnostics(self) -> dict:
        """diagnostics() (src/core/model.ts:1672-1696) without shear06."""
        d = SgDiagnostics()
        self.ctx.check(load().sg_run_diagnostics(self.ctx.h, self.id, C.byref(d)), "diagnostics")
        return {k: getattr(d, k) for k, _ in SgDiagnostics._fields_}

    def save_state(self, config: Optional[dict] = None, persisted: Optional[float] = None) -> bytes:
        """saveState (src/core/state.ts:43-53): the run as a .meteolab image, at this run's model time; `persisted`
        defaults to the device's own count when the run tracks its rotation (else 0)."""
        if persisted is None:
            persisted = self.rotation()["persisted"] if self.spec.switches.rotation else 0.0
        cfg = json.dumps(config, separators=(",", ":")).encode() if config is not None else None
        size = C.c_size_t()
        self.ctx.check(load().sg_run_save_state(self.ctx.h, self.id, cfg, self.time, persisted, None, 0, C.byref(size)), "save state")
        buf = C.create_string_buffer(size.value)
        self.ctx.check(load().sg_run_save_state(self.ctx.h, self.id, cfg, self.time, persisted, buf, size.value, C.byref(size)),
                       "save state")
        return buf.raw[:size.value]

    def load_state(self, image: bytes) -> dict:
        """readState + applyState (src/core/state.ts:55-83): the image's fields and columns into this run; the run's
        model time becomes the file's."""
        info = SgStateInfo()
        self.ctx.check(load().sg_run_load_state(self.ctx.h, self.id, image, len(image), C.byref(info)), "load state")
        self.time = info.time
        return _info_dict(info)


def _info_dict(info: "SgStateInfo") -> dict:
    return {k: getattr(info, k) for k, _ in SgStateInfo._fields_ if k != "reserved"}


def parse_state(image: bytes) -> dict:
    """readState's checks alone (sg_state_parse; no context, no device): the header's values, or StormGpuError with
    the reference's message."""
    info = SgStateInfo()
    err = C.create_string_buffer(200)
    rc = load().sg_state_parse(image, len(image), C.byref(info), err, len(err))
    if rc:
        raise StormGpuError(rc, err.value.decode())
    return _info_dict(info)


class AtmosphereModel:
    """The reference's model interface (src/core/model.ts:183-210, :873) over one device run: ``step(dt)`` advances
    by one model step and moves ``time`` (the reference's callers add dt themselves, src/core/fixtures.ts:28-30);
    the fields read back as FP32 arrays in node order."""

    def __init__(self, spec: RunSpec, context: Optional[Context] = None):
        self.context = context or Context()
        self.spec, self.grid, self.env = spec, spec.grid, spec.env
        self.run = self.context.create(spec)
        self.time = 0.0

    def step(self, dt: Optional[float] = None):
        if dt is not None and abs(dt - self.spec.switches.dt) > 1e-12:
            raise StormGpuError(1, f"the run was set up for dt = {self.spec.switches.dt}")
        self.run.step(1)
        self.time += self.spec.switches.dt

    def __getattr__(self, name):
        if name in CARRIED:
            return self.run.read([name])[name]
        if name in ("precipitation", "hailGround", "hailSize"):
            return self.run.columns()[name]
        if name == "pressure":
            return self.run.pressure()
        raise AttributeError(name)

    @property
    def clipped(self) -> int:
        return self.run.status()["clipped"]

    @property
    def negativeFilled(self) -> float:
        return self.run.status()["negative_filled"]


class Server:
    """The serving loop (sg_server_*): submit requests, iterate; each iteration admits by HBM budget, advances every
    active run one step in one batch and retires finished runs."""

    def __init__(self, ctx: Context, max_active: int = 256):
        h = C.c_void_p()
        ctx.check(load().sg_server_create(ctx.h, max_active, C.byref(h)), "server create")
        self.ctx, self.h = ctx, h

    def set_quantum(self, steps: int):
        """Advance up to `steps` steps per iteration (stopping where the first active run finishes)."""
        self.ctx.check(load().sg_server_set_quantum(self.h, steps), "quantum")

    @property
    def last_steps(self) -> int:
        return load().sg_server_last_steps(self.h)

    def submit(self, spec: RunSpec, steps: int, tag: int):
        p = _Packed(spec)
        self.ctx.check(load().sg_server_submit(self.h, C.byref(p.grid), C.byref(p.base), C.byref(p.switches), p.ptrs, steps, tag), "submit")

    def iterate(self, cap: int = 1024):
        tags = (C.c_int64 * cap)()
        done, active, queued = C.c_int(), C.c_int(), C.c_int()
        self.ctx.check(load().sg_server_iterate(self.h, tags, C.byref(done), cap, C.byref(active), C.byref(queued)), "iterate")
        return [tags[k] for k in range(done.value)], active.value, queued.value

    def collect(self, tag: int, n: int, names: Iterable[str] = CARRIED) -> Dict[str, np.ndarray]:
        """Read a finished run's fields (n nodes each) and retire it."""
        names = list(names)
        out = {k: np.empty(n, np.float32) for k in names}
        ptrs = (_FP * len(CARRIED))()
        mask = 0
        for k in names:
            mask |= 1 << CARRIED.index(k)
            ptrs[CARRIED.index(k)] = out[k].ctypes.data_as(_FP)
        self.ctx.check(load().sg_server_collect(self.h, tag, mask, ptrs, None), "collect")
        return out

    def close(self):
        if getattr(self, "h", None):
            load().sg_server_destroy(self.h)
            self.h = None


class ElectricSolver:
    """The storm's electric potential on the device, the reference's ElectricSolver (src/core/electric.ts:15-72):
    ``solve(rho)`` returns phi (V) with Laplacian(phi) = -rho/eps0 at the nodes (rho in C/m3, nx*ny*nz values), phi = 0
    on the ground and top levels, periodic in x and y; ``field(phi, x, y, z)`` is E = -grad(phi) at a node."""

    def __init__(self, ctx: Context, grid):
        self.ctx, self.grid = ctx, grid
        self._keep = [_f64(grid.zs), _f64(grid.dzs), _f64(grid.hz)]
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        g = SgGrid(grid.nx, grid.ny, grid.nz, 0, grid.dx, grid.dy, grid.height, dp(self._keep[0]), dp(self._keep[1]), dp(self._keep[2]))
        h = C.c_void_p()
        ctx.check(load().sg_electric_create(ctx.h, C.byref(g), C.byref(h)), "electric solver")
        self.h = h

    def solve(self, rho: np.ndarray, out: Optional[np.ndarray] = None) -> np.ndarray:
        n = self.grid.nx * self.grid.ny * self.grid.nz
        rho = np.ascontiguousarray(rho, dtype=np.float64).ravel()
        if rho.size != n:
            raise ValueError(f"rho must hold {n} values")
        phi = out if out is not None else np.empty(n, np.float64)
        if phi.dtype != np.float64 or not phi.flags.c_contiguous or phi.size != n:
            raise ValueError(f"phi must be a contiguous float64 array of {n}")
        self.ctx.check(load().sg_electric_solve(self.h, rho.ctypes.data_as(C.POINTER(C.c_double)), phi.ctypes.data_as(C.POINTER(C.c_double))),
                       "electric solve")
        return phi

    def field(self, phi: np.ndarray, x: int, y: int, z: int):
        """E = -grad(phi) (V/m) at node (x, y, z): centred, periodic in x and y, one-sided at the ground and top (:64-71)."""
        g = self.grid
        nx, ny, nz, layer = g.nx, g.ny, g.nz, g.nx * g.ny

        def at(i, j, k):
            return phi[((i + nx) % nx) + ((j + ny) % ny) * nx + k * layer]
        lo, hi = max(0, z - 1), min(nz - 1, z + 1)
        return (-(at(x + 1, y, z) - at(x - 1, y, z)) / (2 * g.dx), -(at(x, y + 1, z) - at(x, y - 1, z)) / (2 * g.dy),
                -(at(x, y, hi) - at(x, y, lo)) / (g.zs[hi] - g.zs[lo]))

    def close(self):
        if getattr(self, "h", None):
            load().sg_electric_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


TERRAIN_KINDS = {"hill": 0, "ridge": 1, "plateau": 2, "schar": 3}


def _grid_struct(grid):
    keep = (_f64(grid.zs), _f64(grid.dzs), _f64(grid.hz))
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    return SgGrid(grid.nx, grid.ny, grid.nz, 0, grid.dx, grid.dy, grid.height, dp(keep[0]), dp(keep[1]), dp(keep[2])), keep


def terrain_heights(terrain: dict, grid) -> np.ndarray:
    """terrainHeights (src/core/terrain.ts:37-63): the ground height of every column, m, float32 [ny*nx], of a terrain
    form as SimConfig.terrain gives it: {kind: 'hill'|'ridge'|'plateau'|'schar', height, width (km), optional x, y (km),
    heading (degrees), wavelength (km)}."""
    nan = float("nan")
    t = SgTerrain(TERRAIN_KINDS[terrain["kind"]], 0, float(terrain["height"]), float(terrain["width"]),
                  *(float(terrain[k]) if terrain.get(k) is not None else nan for k in ("x", "y", "heading", "wavelength")))
    g, keep = _grid_struct(grid)
    out = np.zeros(grid.nx * grid.ny, np.float32)
    if load().sg_terrain_heights(C.byref(g), C.byref(t), out.ctypes.data_as(_FP)) != 0:
        raise StormGpuError(1, "terrain heights: an invalid grid or form")
    return out


def terrain_geometry(grid, ground) -> dict:
    """The cut cells of ground heights (terrain.ts): solidMask, groundLevels, nodeHeights, faceApertures (ax, ay) and
    slopeArea, computed by the library on the host."""
    g, keep = _grid_struct(grid)
    h = np.ascontiguousarray(ground, dtype=np.float32)
    n, layer = grid.nx * grid.ny * grid.nz, grid.nx * grid.ny
    if h.size != layer:
        raise ValueError(f"ground must hold {layer} heights")
    out = {"solid": np.zeros(n, np.uint8), "levels": np.zeros(layer, np.int32), "heights": np.zeros(n), "ax": np.zeros(n),
           "ay": np.zeros(n), "slope": np.zeros(layer, np.float32)}
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    if load().sg_terrain_geometry(C.byref(g), h.ctypes.data_as(_FP), out["solid"].ctypes.data_as(C.POINTER(C.c_uint8)),
                                  out["levels"].ctypes.data_as(C.POINTER(C.c_int32)), dp(out["heights"]), dp(out["ax"]), dp(out["ay"]),
                                  out["slope"].ctypes.data_as(_FP)) != 0:
        raise StormGpuError(1, "terrain geometry: an invalid grid or ground")
    return out


class MaskedProjection:
    """The reference's MaskedProjection (src/core/terrain.ts:168-363) on the device: ``project(u, v, w, dt, pressure)``
    makes the node mass flux rho0 u divergence-free over the dual cells cut by the ground, in place, by preconditioned
    conjugate gradients around the flat spectral solve; ``pressure`` (nx*ny*(nz-1) cells) is the first guess and gets
    the result. ``mask``, ``divergence``, ``iterations``, ``residual`` and ``dropped`` as the reference's."""

    def __init__(self, ctx: Context, grid, rho, ground, tolerance: float = 1e-6, max_iterations: int = 200):
        self.ctx, self.grid = ctx, grid
        self._g, self._keep = _grid_struct(grid)
        r = _f64(rho)
        h = np.ascontiguousarray(ground, dtype=np.float32)
        if r.size != grid.nz or h.size != grid.nx * grid.ny:
            raise ValueError(f"rho needs {grid.nz} levels and ground {grid.nx * grid.ny} columns")
        hnd = C.c_void_p()
        ctx.check(load().sg_masked_create(ctx.h, C.byref(self._g), r.ctypes.data_as(C.POINTER(C.c_double)), h.ctypes.data_as(_FP),
                                          tolerance, max_iterations, C.byref(hnd)), "masked projection")
        self.h = hnd
        self.cells = grid.nx * grid.ny * (grid.nz - 1)

    def _fields(self, *arrays):
        n = self.grid.nx * self.grid.ny * self.grid.nz
        for a in arrays:
            if a.dtype != np.float32 or not a.flags.c_contiguous or a.size != n:
                raise ValueError(f"u, v and w must be contiguous float32 arrays of {n}")
        return [a.ctypes.data_as(_FP) for a in arrays]

    def project(self, u: np.ndarray, v: np.ndarray, w: np.ndarray, dt: float, pressure: np.ndarray) -> None:
        if pressure.dtype != np.float64 or not pressure.flags.c_contiguous or pressure.size != self.cells:
            raise ValueError(f"pressure must be a contiguous float64 array of {self.cells}")
        self.ctx.check(load().sg_masked_project(self.h, *self._fields(u, v, w), dt, pressure.ctypes.data_as(C.POINTER(C.c_double))),
                       "masked projection")

    def mask(self, u: np.ndarray, v: np.ndarray, w: np.ndarray) -> None:
        self.ctx.check(load().sg_masked_mask(self.h, *self._fields(u, v, w)), "masked projection")

    def divergence(self, u: np.ndarray, v: np.ndarray, w: np.ndarray, out: Optional[np.ndarray] = None) -> np.ndarray:
        out = np.empty(self.cells) if out is None else out
        self.ctx.check(load().sg_masked_divergence(self.h, *self._fields(u, v, w), out.ctypes.data_as(C.POINTER(C.c_double))),
                       "masked projection")
        return out

    @property
    def iterations(self) -> int:
        it = C.c_int32()
        load().sg_masked_stats(self.h, C.byref(it), None)
        return int(it.value)

    @property
    def residual(self) -> float:
        r = C.c_double()
        load().sg_masked_stats(self.h, None, C.byref(r))
        return float(r.value)

    @property
    def dropped(self) -> np.ndarray:
        out = np.zeros(self.cells, np.uint8)
        load().sg_masked_dropped(self.h, out.ctypes.data_as(C.POINTER(C.c_uint8)))
        return out

    def close(self):
        if getattr(self, "h", None):
            load().sg_masked_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class TerrainFaces:
    """The reference's transport faces with terrain (FluxTransport.setTerrain and setVelocityMasked,
    src/core/advection.ts:78-184) on the device: ``set_velocity_masked(u, v, w)`` returns the face mass fluxes
    (mx, my, mz) of the node velocity, shut next to the ground and divergence-free over the fluid nodes with the faces'
    open heights, and their divergence over the node heights (div); ``iterations`` and ``residual`` as the reference's
    maskedIterations and maskedResidual."""

    def __init__(self, ctx: Context, grid, rho, ground, tolerance: float = 1e-10, max_iterations: int = 400):
        self.ctx, self.grid = ctx, grid
        self._g, self._keep = _grid_struct(grid)
        r = _f64(rho)
        h = np.ascontiguousarray(ground, dtype=np.float32)
        if r.size != grid.nz or h.size != grid.nx * grid.ny:
            raise ValueError(f"rho needs {grid.nz} levels and ground {grid.nx * grid.ny} columns")
        hnd = C.c_void_p()
        ctx.check(load().sg_faces_create(ctx.h, C.byref(self._g), r.ctypes.data_as(C.POINTER(C.c_double)), h.ctypes.data_as(_FP),
                                         tolerance, max_iterations, C.byref(hnd)), "masked faces")
        self.h = hnd

    def set_velocity_masked(self, u: np.ndarray, v: np.ndarray, w: np.ndarray):
        n = self.grid.nx * self.grid.ny * self.grid.nz
        fields = [np.ascontiguousarray(a, dtype=np.float32) for a in (u, v, w)]
        if any(a.size != n for a in fields):
            raise ValueError(f"u, v and w must hold {n} values")
        out = [np.empty(n) for _ in range(4)]
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        self.ctx.check(load().sg_faces_set_velocity(self.h, *[a.ctypes.data_as(_FP) for a in fields], *[dp(a) for a in out]), "masked faces")
        return tuple(out)

    @property
    def iterations(self) -> int:
        it = C.c_int32()
        load().sg_faces_stats(self.h, C.byref(it), None)
        return int(it.value)

    @property
    def residual(self) -> float:
        r = C.c_double()
        load().sg_faces_stats(self.h, None, C.byref(r))
        return float(r.value)

    def close(self):
        if getattr(self, "h", None):
            load().sg_faces_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def divergence_max_static(device: int, u_ptr: int, v_ptr: int, w_ptr: int, grid, rho, stream: int = 0) -> float:
    """Max |D rho0 u| of velocity fields already in device memory (raw device pointers, nx*ny*nz FP32 each), without
    any allocation by the library (sg_divergence_max_static)."""
    rho = _f64(rho)
    dzs = _f64(grid.dzs)
    if rho.size < grid.nz or dzs.size < grid.nz - 1:
        raise ValueError(f"rho needs {grid.nz} levels and dzs {grid.nz - 1} spacings (got {rho.size}, {dzs.size})")
    out = C.c_double()
    err = C.create_string_buffer(160)
    rc = load().sg_divergence_max_static(device, u_ptr, v_ptr, w_ptr, grid.nx, grid.ny, grid.nz, grid.dx, grid.dy,
                                         rho.ctypes.data_as(C.POINTER(C.c_double)), dzs.ctypes.data_as(C.POINTER(C.c_double)),
                                         stream or None, C.byref(out), err, len(err))
    if rc:
        raise StormGpuError(rc, err.value.decode())
    return out.value
