"""Base state of a run: the horizontally uniform environment per level (host-side set-up of the step).

Restates ``Environment`` (src/core/environment.ts:32-58), its hydrostatic integration (:64-73), the slider profile
(:86-184) and the analytic ``weismanKlemp`` profile (src/core/profiles.ts:61-73). The per-level arrays it produces
(p, exner, theta, q, u, v, rho; FP64) are what the C ABI's ``sg_base_state`` carries to the device.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, Optional, Tuple

import numpy as np

from .grid import Grid

# src/core/constants.ts:1-6
G, CP, LV, KAPPA, RD, RV, EPS, OMEGA = 9.81, 1004.0, 2.5e6, 0.286, 287.05, 461.5, 0.622, 7.2921e-5
DT = 3.0

SURFACE_PRESSURE, PRESSURE_STEP = 101325.0, 10.0
CAP_DEPTH, CAP_FADE = 300.0, 2000.0
NIGHT_DEPTH, RESIDUAL_COOLING = 400.0, 0.25
NEUTRAL_STEP = 10.0


def clamp(x: float, a: float = 0.0, b: float = 1.0) -> float:
    return max(a, min(b, x))


def lerp(a: float, b: float, t: float) -> float:
    return a + (b - a) * clamp(t)


def mod(x: float, n: float) -> float:
    return ((x % n) + n) % n


def lerp_angle(a: float, b: float, t: float) -> float:
    return mod(a + (mod(b - a + 180, 360) - 180) * clamp(t), 360)


def qsat_p(t: float, p: float) -> float:
    """Saturation mixing ratio over water, t in C, p in Pa (src/core/microphysics.ts:5)."""
    es = 611.2 * math.exp(17.67 * t / (t + 243.5))
    return clamp(EPS * es / max(1000.0, p - es), 0.0, 0.045)


@dataclass
class EnvironmentProfile:
    """An analytic environment (src/core/environment.ts:19-29): theta(z), rh(z), wind(z), optional qv cap."""
    theta: Callable[[float], float]
    rh: Callable[[float], float]
    wind: Callable[[float], Tuple[float, float]]
    qv_max: Optional[float] = None
    qv: Optional[Callable[[float], float]] = None
    surface_pressure: Optional[float] = None


def weisman_klemp(radius: float = 8.0, u6: float = 30.0, qv_max: float = 0.014,
                  depth: Optional[float] = None,
                  wind: Optional[Callable[[float], Tuple[float, float]]] = None) -> EnvironmentProfile:
    """Weisman & Klemp (1982) sounding (src/core/profiles.ts:61-73); ``wind`` replaces the hodograph if given."""
    ztr, theta_tr, t_tr = 12_000.0, 343.0, 213.0

    def theta(z: float) -> float:
        return 300 + (theta_tr - 300) * (z / ztr) ** 1.25 if z <= ztr else theta_tr * math.exp(G * (z - ztr) / (CP * t_tr))

    def rh(z: float) -> float:
        return 1 - 0.75 * (z / ztr) ** 1.25 if z <= ztr else 0.25

    def hodograph(z: float) -> Tuple[float, float]:
        if depth:
            return (u6 * min(1.0, z / depth), 0.0)
        if z < 2000:
            a = math.pi / 2 * z / 2000
            return (radius - radius * math.cos(a), radius * math.sin(a))
        return (radius + (u6 - radius) * min(1.0, (z - 2000) / 4000), radius)

    return EnvironmentProfile(theta, rh, wind or hodograph, qv_max)


def tanh_shear(top_speed: float = 20.0, scale: float = 3000.0, veer_deg: float = 0.0):
    """The wind u = U tanh(z / scale), turned by up to ``veer_deg`` degrees clockwise from the ground upwards."""
    def wind(z: float) -> Tuple[float, float]:
        s = top_speed * math.tanh(z / scale)
        turn = math.radians(veer_deg) * min(1.0, z / 6000.0)
        return (s * math.cos(turn), -s * math.sin(turn))
    return wind


@dataclass
class SliderConfig:
    """The slider-profile part of ``SimConfig`` (src/core/config.ts:15-20, 26-34) with the SUMMER_DAY values
    (src/core/fixtures.ts:6-12)."""
    surfaceTemp: float = 30
    lapseLow: float = 8.4
    lapseMid: float = 7.2
    lapseUpper: float = 6.5
    tropopause: float = 11
    stratoWarming: float = 1.2
    rhSurface: float = 72
    rhLow: float = 60
    rhMid: float = 42
    rhUpper: float = 28
    wind0: float = 2
    wind3: float = 10
    wind6: float = 20
    wind10: float = 28
    windDir0: float = 160
    windDir3: float = 185
    windDir6: float = 215
    windDir10: float = 235
    wind05: Optional[float] = None
    windDir05: Optional[float] = None
    wind1: Optional[float] = None
    windDir1: Optional[float] = None
    capHeight: Optional[float] = None
    capStrength: Optional[float] = None
    nightInversion: Optional[float] = None
    moistLayer: Optional[float] = None


class Environment:
    """Per-level base state (src/core/environment.ts:32-58)."""

    def __init__(self, config: SliderConfig, grid: Grid, profile: Optional[EnvironmentProfile] = None):
        self.config, self.profile = config, profile
        self.neutral: Optional[np.ndarray] = None
        self.lnP = self._integrate_hydrostatic(grid.height + 2000)
        if profile is None:
            for _ in range(2):
                self.neutral = self._neutralise(grid.height + 2000)
                self.lnP = self._integrate_hydrostatic(grid.height + 2000)
        nz = grid.nz
        self.p, self.exner, self.theta = np.zeros(nz), np.zeros(nz), np.zeros(nz)
        self.q, self.u, self.v, self.rho = np.zeros(nz), np.zeros(nz), np.zeros(nz), np.zeros(nz)
        for z in range(nz):
            alt = float(grid.zs[z])
            u, v = self.wind_uv(alt)
            self.p[z] = self.pressure_at(alt)
            self.exner[z] = (self.p[z] / 100000) ** KAPPA
            self.theta[z] = self.theta_env(alt)
            self.q[z] = self.q_env(alt)
            self.u[z], self.v[z] = u, v
            self.rho[z] = self.p[z] / (RD * self.theta[z] * self.exner[z] * (1 + 0.61 * self.q[z]))

    @classmethod
    def winds_only(cls, config: SliderConfig) -> "Environment":
        """An environment that answers only for its wind (the slider's nodes), without the base state's integration."""
        e = cls.__new__(cls)
        e.config, e.profile, e.neutral = config, None, None
        return e

    # -- hydrostatic pressure (src/core/environment.ts:64-78)
    def _integrate_hydrostatic(self, top: float) -> np.ndarray:
        n = math.ceil(top / PRESSURE_STEP) + 1
        ln_p = np.zeros(n)
        ln_p[0] = math.log(self.profile.surface_pressure if self.profile and self.profile.surface_pressure
                           else SURFACE_PRESSURE)

        def tv(z: float, p: float) -> float:
            t = self._temperature_at(z, p)
            q = self.mixing_ratio(z, t, p)
            return (t + 273.15) * (1 + 0.61 * q)

        for k in range(n - 1):
            z = k * PRESSURE_STEP
            p = math.exp(ln_p[k])
            ln_p[k + 1] = ln_p[k] - G * PRESSURE_STEP / (RD * 0.5 * (tv(z, p) + tv(z + PRESSURE_STEP, p)))
        return ln_p

    def pressure_at(self, z: float) -> float:
        ln_p = self.lnP
        x = max(0.0, z) / PRESSURE_STEP
        k = min(math.floor(x), len(ln_p) - 2)
        return math.exp(ln_p[k] + (ln_p[k + 1] - ln_p[k]) * (x - k))

    # -- temperature (src/core/environment.ts:80-147)
    def temperature_env(self, z: float) -> float:
        return self._temperature_at(z, self.pressure_at(z)) if self.profile else self._slider_temperature(z)

    def _temperature_at(self, z: float, p: float) -> float:
        if self.profile:
            return self.profile.theta(z) * (p / 100000) ** KAPPA - 273.15
        return self._slider_temperature(z)

    def _slider_temperature(self, z: float) -> float:
        return self._day_temperature(z) - self.night_deficit(z) + self._neutral_warmth(z)

    def _neutral_warmth(self, z: float) -> float:
        n = self.neutral
        if n is None:
            return 0.0
        x = min(max(0.0, z) / NEUTRAL_STEP, len(n) - 1.001)
        k = math.floor(x)
        return float(n[k] + (n[k + 1] - n[k]) * (x - k))

    def _neutralise(self, top: float) -> np.ndarray:
        n = math.ceil(top / NEUTRAL_STEP) + 2
        warmth = np.zeros(n, dtype=np.float32)
        level = 0.0
        for k in range(n):
            z = k * NEUTRAL_STEP
            p = self.pressure_at(z)
            pi = (100000 / p) ** KAPPA
            plain = self._day_temperature(z) - self.night_deficit(z)
            moist = pi * (1 + 0.61 * self._q_at(z, plain, p))
            thv = (plain + 273.15) * moist
            warmth[k] = max(0.0, (level - thv) / moist)
            level = max(level, thv)
        return warmth

    def night_deficit(self, z: float) -> float:
        n = 0 if self.profile else (self.config.nightInversion or 0)
        if not n > 0:
            return 0.0
        top = max(NIGHT_DEPTH, (self.config.capHeight if self.config.capHeight is not None else 1.5) * 1000)
        if z < NIGHT_DEPTH:
            return n * (1 - (1 - RESIDUAL_COOLING) * z / NIGHT_DEPTH)
        return n * RESIDUAL_COOLING * max(0.0, min(1.0, 1 - (z - top) / NIGHT_DEPTH))

    def _day_temperature(self, z: float) -> float:
        c = self.config
        strength = c.capStrength or 0
        if not strength > 0:
            return self._lapse_temperature(z)
        base = (c.capHeight if c.capHeight is not None else 1.5) * 1000
        top = base + CAP_DEPTH
        bump = strength + self._lapse_temperature(base) - self._lapse_temperature(top)
        f = 0.0 if z <= base else (z - base) / CAP_DEPTH if z < top else max(0.0, 1 - (z - top) / CAP_FADE)
        return self._lapse_temperature(z) + bump * f

    def _lapse_temperature(self, z: float) -> float:
        c = self.config
        tp = c.tropopause * 1000
        t3 = c.surfaceTemp - c.lapseLow * 3
        t8 = t3 - c.lapseMid * 5
        if z <= 3000:
            return c.surfaceTemp - c.lapseLow * z / 1000
        if z <= 8000:
            return t3 - c.lapseMid * (z - 3000) / 1000
        ttp = t8 - c.lapseUpper * (tp - 8000) / 1000
        if z <= tp:
            return t8 - c.lapseUpper * (z - 8000) / 1000
        return ttp + c.stratoWarming * (z - tp) / 1000

    def theta_env(self, z: float) -> float:
        return (self.temperature_env(z) + 273.15) * (100000 / self.pressure_at(z)) ** KAPPA

    # -- humidity (src/core/environment.ts:151-184)
    def rh_env(self, z: float) -> float:
        if self.profile:
            return self.profile.rh(z)
        c = self.config
        tp = c.tropopause * 1000
        if z < 1500:
            return lerp(c.rhSurface, c.rhLow, z / 1500) / 100
        if z < 5000:
            return lerp(c.rhLow, c.rhMid, (z - 1500) / 3500) / 100
        if z < tp:
            return lerp(c.rhMid, c.rhUpper, (z - 5000) / max(1000.0, tp - 5000)) / 100
        return c.rhUpper / 100 * 0.7

    def q_env(self, z: float) -> float:
        return self._q_at(z, self.temperature_env(z) - self._neutral_warmth(z), self.pressure_at(z))

    def _q_at(self, z: float, t: float, p: float) -> float:
        d = self.night_deficit(z)
        if not d:
            return self.mixing_ratio(z, t, p)
        residual = min(d, (self.config.nightInversion or 0) * RESIDUAL_COOLING)
        day = t + d
        return min(self.mixing_ratio(z, day, p) * qsat_p(day - residual, p) / qsat_p(day, p), 0.97 * qsat_p(t, p))

    def mixing_ratio(self, z: float, t: float, p: float) -> float:
        if self.profile and self.profile.qv:
            return min(self.profile.qv(z), qsat_p(t, p))
        cap = self.profile.qv_max if self.profile and self.profile.qv_max is not None else math.inf
        r = min(self.rh_env(z) * qsat_p(t, p), cap)
        top = (self.config.moistLayer or 0) * 1000
        if self.profile or z >= top:
            return r
        surface = self.config.rhSurface / 100 * qsat_p(self.config.surfaceTemp, SURFACE_PRESSURE)
        return min(max(r, surface), qsat_p(t, p))

    # -- wind (src/core/environment.ts:187-212)
    def _wind_nodes(self):
        c = self.config
        nodes = [(0.0, c.wind0, c.windDir0)]
        if c.wind05 is not None and c.windDir05 is not None:
            nodes.append((500.0, c.wind05, c.windDir05))
        if c.wind1 is not None and c.windDir1 is not None:
            nodes.append((1000.0, c.wind1, c.windDir1))
        nodes += [(3000.0, c.wind3, c.windDir3), (6000.0, c.wind6, c.windDir6), (10000.0, c.wind10, c.windDir10)]
        return nodes

    def _wind_at(self, z: float, component: int) -> float:
        nodes = self._wind_nodes()
        interp = lerp if component == 1 else lerp_angle
        for k in range(1, len(nodes)):
            if z < nodes[k][0]:
                a, b = nodes[k - 1], nodes[k]
                return interp(a[component], b[component], (z - a[0]) / (b[0] - a[0]))
        top = nodes[-1][component]
        return top if component == 1 else mod(top, 360)

    def wind_uv(self, z: float) -> Tuple[float, float]:
        if self.profile:
            return self.profile.wind(z)
        s = self._wind_at(z, 1)
        a = (270 - self._wind_at(z, 2)) * math.pi / 180
        return (s * math.cos(a), s * math.sin(a))

    def wind_scalar(self, z: float) -> float:
        return self._wind_at(z, 1)

    def wind_direction(self, z: float) -> float:
        """Direction the wind blows from, turning along the shorter arc between the nodes (environment.ts:201)."""
        return self._wind_at(z, 2)

    def qsat(self, t: float, z: float) -> float:
        return qsat_p(t, self.pressure_at(z))

    def dewpoint(self, q: float, z: float) -> float:
        """Dew point, C, of mixing ratio q at height z (environment.ts:214)."""
        e = max(1.0, q * self.pressure_at(z) / (EPS + q))
        lg = math.log(e / 611.2)
        return 243.5 * lg / (17.67 - lg)

    def base_state(self) -> dict:
        """The per-level arrays the device needs (FP64)."""
        return dict(p=self.p.copy(), exner=self.exner.copy(), theta=self.theta.copy(), q=self.q.copy(),
                    u=self.u.copy(), v=self.v.copy(), rho=self.rho.copy())
