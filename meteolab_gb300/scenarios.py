"""Run set-up: switches, seeded soundings and initial states of the benchmark workloads.

The switches mirror the model defaults of ``AtmosphereModel`` (src/core/model.ts:747-844) with the SUMMER_DAY
configuration (src/core/fixtures.ts:6-12): WENO transport, ice microphysics (one-moment), anisotropic Smagorinsky
width, explicit vertical mixing, theta-e moist stability, pressure in the RK3 stages, wind relaxation 1e-4 1/s,
sponge 0.06 1/s. The single-storm mode (``single``: no sun, no surface pattern, src/core/config.ts:147-152) is the
only surface mode the device step supports.

Initial state: the ``ellipsoid`` start (src/core/model.ts:94, :431-437) with the amplitude as a parameter, plus
seeded uniform noise below a height, drawn with ``mulberry32`` (src/core/math.ts:7-14) in node order.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, asdict
from typing import Dict, List, Optional, Tuple

import numpy as np

from .environment import (CP, G, OMEGA, Environment, EnvironmentProfile, SliderConfig, tanh_shear, weisman_klemp)
from .grid import Grid

#: The transported fields in the order the step carries them (src/core/model.ts:1319-1335, ice on, no lightning).
CARRIED = ("rain", "snow", "graupel", "hail", "u", "v", "w", "theta", "q", "cloud", "ice", "iceNumber", "cold")
# the charge carriers of an electrified run, C/kg (field ids 13-16 of the C ABI; src/core/model.ts:210)
CHARGES = ("chargeIce", "chargeGraupel", "chargeRain", "chargeAir")
# two-moment graupel and hail (src/core/model.ts:202): particles per kg and particle volume, m3 per kg
ICE2M = ("graupelNumber", "graupelVolume", "hailNumber", "hailVolume")
#: The fields the subgrid turbulence mixes (src/core/model.ts:1338-1344).
MIXED = ("u", "v", "w", "theta", "q", "cloud", "ice", "iceNumber")
SMAGORINSKY = 0.18
SURFACE_ROUGHNESS = {"grass": 0.03, "dry": 0.01, "water": 0.0002, "urban": 1.0}


def mulberry32(seed: int):
    """The reference's seeded generator (src/core/math.ts:7-14), 32-bit integer semantics of JS."""
    state = [seed & 0xFFFFFFFF]

    def imul(a: int, b: int) -> int:
        return (a * b) & 0xFFFFFFFF

    def nxt() -> float:
        s = (state[0] + 0x6D2B79F5) & 0xFFFFFFFF
        state[0] = s
        t = imul(s ^ (s >> 15), 1 | s)
        t = ((t + imul(t ^ (t >> 7), 61 | t)) & 0xFFFFFFFF) ^ t
        return ((t ^ (t >> 14)) & 0xFFFFFFFF) / 4294967296.0

    return nxt


def drag_coefficient(surface: str, dz: float) -> float:
    """Neutral drag coefficient of the ground node (src/core/surface.ts:9)."""
    return (0.4 / math.log(dz / 4 / SURFACE_ROUGHNESS[surface])) ** 2


@dataclass
class Switches:
    """Scalar settings of a run: the POD ``sg_switches`` of the C ABI (field for field)."""
    dt: float = 3.0
    coriolis: float = 2 * OMEGA * math.sin(45 * math.pi / 180)  # f at SUMMER_DAY's latitude 45
    wind_relaxation: float = 1e-4
    sponge_rate: float = 0.06
    sponge_start: float = 14_000.0  # max(tropopause*1000 + 2500, 14 km) with tropopause 11 km
    cs: float = SMAGORINSKY         # SMAGORINSKY * turbulence / .55 with the default slider .55
    drag: float = 1.0               # 1: surface drag on (coefficient from the surface type), 0: off
    surface: str = "grass"
    frame_u: float = 0.0
    frame_v: float = 0.0
    loading: int = 1
    evaporation: int = 1
    rain_formation: int = 1
    anisotropic: int = 1
    vertical_dz: int = 0
    durran_klemp: int = 0
    pressure_in_stages: int = 1
    # the device refines its final projection once (FP32-transform residual solved again); the oracle's FP64 solve
    # needs no refinement and ignores it
    refine_projection: int = 1
    rotation: int = 1   # the rotation tracking after every step (afterStep) and the swaths, on the device
    ice: int = 1        # the ice microphysics (the warm scheme when 0)
    # electrification and lightning (SimConfig.lightning; with the ice microphysics only, src/core/model.ts:1316): the
    # four charge carriers, the charging in the physics and the flashes after every step; corona from the ground (over
    # land, not over water); the lightning's seed (config.seed + 1, :1538)
    lightning: int = 0
    corona: int = 1
    lightning_seed: int = 43
    # two-moment rain (AtmosphereModel.rainMoments 2, src/core/model.ts:842): the raindrop number carried with the rain;
    # its collisional breakup 0 none (the default), 1 NSSL's, 2 Morrison's (:843, src/core/rain2m.ts:23-31)
    rain_moments: int = 1
    rain_breakup: int = 0
    # two-moment graupel and hail (AtmosphereModel.iceMoments 2, src/core/model.ts:839-840; with the ice microphysics and
    # two-moment rain only, :914): their number and particle volume carried with their mass (src/core/ice2m.ts)
    ice_moments: int = 1

    def drag_cd(self, grid: Grid) -> float:
        return drag_coefficient(self.surface, 2 * float(grid.hz[0])) if self.drag else 0.0


@dataclass
class RunSpec:
    """Everything that defines one run: its grid, environment, switches and initial fields."""
    grid: Grid
    env: Environment
    switches: Switches
    fields: Dict[str, np.ndarray]
    seed: int = 0
    label: str = ""
    meta: Dict[str, float] = field(default_factory=dict)   # what a workload records about the run (CAPE, shear, lid)

    @property
    def cells(self) -> int:
        return self.grid.n


def baseline_profile(qv_max: float = 0.014, shear: float = 20.0, veer: float = 0.0) -> EnvironmentProfile:
    """The analytic benchmark sounding: Weisman-Klemp theta and RH, qv capped, wind ``shear * tanh(z / 3 km)``."""
    return weisman_klemp(qv_max=qv_max, wind=tanh_shear(shear, 3000.0, veer))


def initial_fields(grid: Grid, env: Environment, seed: int, bubble: float = 2.0, noise: float = 0.1,
                   noise_top: float = 1000.0, frame: Tuple[float, float] = (0.0, 0.0),
                   across: float = 1 / 3) -> Dict[str, np.ndarray]:
    """Initial fields: environment profile, a cos^2 ellipsoid bubble (radii 10 km / 1.4 km at 1.4 km, a third of the
    way in from the west, src/core/model.ts:94), uniform noise of +-``noise`` K below ``noise_top``; FP32 like the
    reference's ``Float32Array`` fields."""
    nx, ny, nz = grid.nx, grid.ny, grid.nz
    zs = grid.zs
    rng = mulberry32(seed)
    theta = np.empty((nz, ny, nx))
    q = np.empty((nz, ny, nx))
    u = np.empty((nz, ny, nx))
    v = np.empty((nz, ny, nx))
    for z in range(nz):
        theta[z] = env.theta[z]
        q[z] = env.q[z]
        u[z] = env.u[z] - frame[0]
        v[z] = env.v[z] - frame[1]
        if zs[z] < noise_top and noise > 0:
            draws = np.array([rng() for _ in range(nx * ny)]).reshape(ny, nx)
            theta[z] += (draws - 0.5) * 2 * noise
    theta32 = theta.astype(np.float32)
    if bubble:
        radius, depth, height = 10_000.0, 1400.0, 1400.0
        x = np.arange(nx) * grid.dx - grid.width * across
        y = np.arange(ny) * grid.dy - grid.depth / 2
        for z in range(nz):
            beta = np.sqrt((x[None, :] / radius) ** 2 + (y[:, None] / radius) ** 2 + ((zs[z] - height) / depth) ** 2)
            inside = beta < 1
            if inside.any():
                add = bubble * np.cos(np.pi * beta / 2) ** 2
                layer = theta32[z].astype(np.float64)
                layer[inside] += add[inside]
                theta32[z] = layer.astype(np.float32)
    zero = np.zeros(grid.n, dtype=np.float32)
    out = {name: zero.copy() for name in CARRIED}
    out["u"] = u.astype(np.float32).ravel()
    out["v"] = v.astype(np.float32).ravel()
    out["theta"] = theta32.ravel()
    out["q"] = q.astype(np.float32).ravel()
    return out


def baseline_run(grid: Grid, seed: int = 42, bubble: float = 2.0, qv_max: float = 0.014, shear: float = 20.0,
                 veer: float = 0.0, switches: Optional[Switches] = None, label: str = "") -> RunSpec:
    """One run of the benchmark configuration on ``grid`` (analytic sounding, single-storm mode)."""
    env = Environment(SliderConfig(), grid, baseline_profile(qv_max, shear, veer))
    sw = switches or Switches()
    fields = initial_fields(grid, env, seed, bubble, frame=(sw.frame_u, sw.frame_v))
    return RunSpec(grid, env, sw, fields, seed, label)


def ensemble_members(grid: Grid, count: int, seed: int = 2026) -> List[RunSpec]:
    """Seeded ensemble members: surface qv U[11, 16] g/kg, 0-6 km shear U[0, 30] m/s with a veering of U[0, 90] deg,
    bubble amplitude U[1, 3] K; each member's own noise seed."""
    rng = np.random.default_rng(seed)
    runs = []
    for k in range(count):
        qv = rng.uniform(0.011, 0.016)
        shear6 = rng.uniform(0.0, 30.0)
        veer = rng.uniform(0.0, 90.0)
        bubble = rng.uniform(1.0, 3.0)
        # tanh(z / 3 km) reaches tanh(2) at 6 km: scale so that the 0-6 km difference is shear6.
        runs.append(baseline_run(grid, seed=seed * 1000 + k, bubble=bubble, qv_max=qv,
                                 shear=shear6 / math.tanh(2.0), veer=veer, label=f"member{k}"))
    return runs


# The regime grid's base settings: the SUMMER_DAY slider profile (src/core/fixtures.ts:6-12) with a well-mixed lowest
# kilometre and the light veering wind of the quiet scenarios (src/core/scenarios.ts:31); its CAPE is set through the
# pair (surface moisture, low-level lapse rate) and its shear by scaling the hodograph about the ground wind.
REGIME_BASE = dict(moistLayer=1.0, wind0=2, wind3=5, wind6=9, wind10=14, windDir0=200, windDir3=230, windDir6=250, windDir10=260)
CAPE_LEVELS = tuple(500.0 + 500.0 * i for i in range(8))   # J/kg, the grid's rows
SHEAR_LEVELS = tuple(40.0 * j / 7 for j in range(8))       # m/s over 0-6 km, the grid's columns


def moisture_lapse(s: float) -> Dict[str, float]:
    """The CAPE knob: s in [0, 1] raises the surface relative humidity (so the boundary layer's vapour) and the
    0-3 km lapse rate together."""
    rh = 40.0 + 25.0 * s
    return dict(rhSurface=rh, rhLow=rh - 5.0, lapseLow=6.0 + 2.0 * s)


def with_shear(values: Dict[str, float], grid: Grid, shear: float) -> Dict[str, float]:
    """The slider hodograph scaled about the ground wind so that the 0-6 km difference is `shear` m/s, its shape kept
    (withShear, src/regime/grid.ts:67-92); a calm hodograph (difference below 2 m/s) gets a straight westerly shear
    added instead."""
    from .environment import SliderConfig
    env = Environment.winds_only(SliderConfig(**values))
    (u0, v0), (u6, v6) = env.wind_uv(0.0), env.wind_uv(6000.0)
    now = math.hypot(u6 - u0, v6 - v0)
    f, added = (shear / now, 0.0) if now > 2 else (1.0, shear)
    out = dict(values)
    for key, z in (("0", 0), ("05", 500), ("1", 1000), ("3", 3000), ("6", 6000), ("10", 10000)):
        speed, direction = values.get(f"wind{key}"), values.get(f"windDir{key}")
        if speed is None or direction is None:
            continue
        a = math.radians(270 - direction)
        u, v = speed * math.cos(a), speed * math.sin(a)
        u, v = u0 + (u - u0) * f + added * min(z, 6000) / 6000, v0 + (v - v0) * f
        out[f"wind{key}"] = math.hypot(u, v)
        if out[f"wind{key}"] > .05:
            out[f"windDir{key}"] = (270 - math.degrees(math.atan2(v, u))) % 360
    return out


def _cape_knob(grid: Grid) -> List[Tuple[float, float]]:
    """Mixed-layer CAPE of the lid-free base profile along the moisture / lapse-rate knob, 11 points."""
    from .environment import SliderConfig
    from .sounding import lift_parcel
    table = []
    for k in range(11):
        env = Environment(SliderConfig(**dict(REGIME_BASE, **moisture_lapse(k / 10))), grid)
        table.append((k / 10, lift_parcel(env, grid.height, "ml").cape))
    return table


def regime_runs(small: Grid, large: Grid, n_small: int = 48, n_large: int = 16, seed: int = 88,
                lid: bool = True) -> List[RunSpec]:
    """An 8 x 8 CAPE x shear regime grid (src/regime/grid.ts) split over two domain sizes.

    Rows: mixed-layer CAPE levels of 500-4000 J/kg, set through the (surface moisture, low-level lapse rate) pair of
    the slider profile (moisture_lapse; the knob's value for each level interpolated from an 11-point table of the
    lid-free profile's CAPE). Columns: 0-6 km shear 0-40 m/s (with_shear). With `lid`, a seeded half of the points
    carries an elevated mixed layer's lid: capStrength U[0, 4] K across the cap law's 300 m at capHeight U[1.5, 3] km
    (src/core/environment.ts:131-138). Each point's own mixed-layer CAPE (lid included) and shear are computed (FP64,
    sounding.py) and kept in its RunSpec's ``meta``. A seeded shuffle puts n_small points on the
    small grid and n_large on the large one; each point has its own bubble amplitude U[1, 3] K and noise seed."""
    from .environment import SliderConfig
    from .sounding import lift_parcel
    rng = np.random.default_rng(seed)
    table = _cape_knob(small)
    ss, cs = [t[0] for t in table], [t[1] for t in table]
    points = [(i, j) for i in range(8) for j in range(8)]
    order = rng.permutation(len(points))
    runs = []
    for slot, p in enumerate(order[:n_small + n_large]):
        i, j = points[p]
        knob = float(np.interp(CAPE_LEVELS[i], cs, ss))
        grid = small if slot < n_small else large
        values = with_shear(dict(REGIME_BASE, **moisture_lapse(knob)), grid, SHEAR_LEVELS[j])
        strength = height = 0.0
        if lid and rng.random() < 0.5:
            strength, height = float(rng.uniform(0.0, 4.0)), float(rng.uniform(1.5, 3.0))
            values.update(capStrength=strength, capHeight=height)
        env = Environment(SliderConfig(**values), grid)
        bubble = float(rng.uniform(1.0, 3.0))
        sd = seed * 1000 + slot
        (u0, v0), (u6, v6) = env.wind_uv(0.0), env.wind_uv(6000.0)
        meta = dict(cape=lift_parcel(env, grid.height, "ml").cape, cape_level=CAPE_LEVELS[i], shear=math.hypot(u6 - u0, v6 - v0),
                    lid_k=strength, lid_km=height)
        runs.append(RunSpec(grid, env, Switches(), initial_fields(grid, env, sd, bubble), sd, f"cape{i}-shear{j}", meta))
    return runs


def serving_requests(small: Grid, large: Grid, count: int, rate: float, seed: int = 5):
    """An open Poisson request stream: arrival times (s) at `rate` runs/s, each request a seeded sounding as the
    ensemble's on the small or the large grid with 3:1 odds, for 20-60 simulated minutes (400-1200 steps of 3 s)."""
    rng = np.random.default_rng(seed)
    t, out = 0.0, []
    for k in range(count):
        t += float(rng.exponential(1.0 / rate))
        grid = small if rng.random() < 0.75 else large
        spec = ensemble_members(grid, 1, seed=seed * 100 + k)[0]
        out.append((t, spec, int(rng.integers(400, 1201))))
    return out


def marshall_palmer_number(rain: np.ndarray, rho: np.ndarray) -> np.ndarray:
    """Raindrops per kg for rain (kg/kg) without a drop number, as two-moment rain starts it (boundedNumber with no
    number, src/core/rain2m.ts:47-51): Marshall-Palmer's N0 / lambda, the mean drop kept between 80 um and a 6 mm
    mass-weighted diameter. `rho` is each node's air density."""
    q = np.asarray(rain, np.float64)
    rho = np.asarray(rho, np.float64)
    out = np.zeros_like(q)
    wet = q > 1e-12
    lam = (math.pi * 1000.0 * 8e6 / (rho[wet] * q[wet])) ** .25
    n = 8e6 / lam / rho[wet]
    xv = np.clip(q[wet] / (1000.0 * n), math.pi / 6 * 80e-6 ** 3, math.pi / 6 * 6e-3 ** 3 / (64 / 6))
    out[wet] = q[wet] / (1000.0 * xv)
    return out.astype(np.float32)


def exponential_ice_moments(q: np.ndarray, rho: np.ndarray, kind: str):
    """Number (per kg) and particle volume (m3 per kg) of two-moment graupel or hail started as the one-moment class of the
    same mass: the exponential distribution of its fixed intercept and density (graupel N0 4e4 m^-4 at 400 kg/m3, hail
    N0 4e4 at 900; src/core/graupel.ts, hail.ts), so the number is N0 / lambda and the volume q / density, as the
    reference's own comparison of the two schemes sets it (ice2m.test.ts:92-98). `rho` is each node's air density."""
    n0, density = {"graupel": (4e4, 400.0), "hail": (4e4, 900.0)}[kind]
    q = np.asarray(q, np.float64)
    rho = np.asarray(rho, np.float64)
    number, volume = np.zeros_like(q), np.zeros_like(q)
    some = q > 1e-12
    lam = (math.pi * density * n0 / (rho[some] * q[some])) ** .25
    number[some] = n0 / lam / rho[some]
    volume[some] = q[some] / density
    return number.astype(np.float32), volume.astype(np.float32)
