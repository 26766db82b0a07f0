"""Parcel indices of a base state (host side, FP64): what the regime grid of the uneven-batch workload reports per
point (its mixed-layer CAPE) and what the environment's known-answer tests check (surface-based CIN).

Restates the reference's parcel ascent (``ascend``, ``moistStep``, ``liftParcel``, ``parcelIndices``:
src/core/sounding.ts:29-68, :71-75, :121-136, :139-160; ``heightOf``, ``thetaE``: :94, :97-100): a parcel lifted in
25 m steps along the environment's pressure, dry adiabat below its lifting condensation level and the pseudo-adiabat
above, CAPE as the net buoyant area between the lowest LFC and the highest EL in virtual temperature (as MetPy).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional

from .environment import CP, EPS, G, KAPPA, LV, RD, Environment, lerp, qsat_p


@dataclass
class Ascent:
    cape: float
    cin: float
    lcl: Optional[float]
    lfc: Optional[float]
    el: Optional[float]
    start: float = 0.0


def moist_step(env: Environment, temp: float, p0: float, p1: float) -> float:
    """One pseudo-adiabatic step of a saturated parcel from pressure p0 to p1, midpoint rule (sounding.ts:71-75)."""
    def dtdp(t: float, p: float) -> float:
        tk = t + 273.15
        rs = qsat_p(t, p)
        return (RD * tk + LV * rs) / (CP + LV * LV * rs * EPS / (RD * tk * tk)) / p
    mid = temp + dtdp(temp, p0) * (p1 - p0) / 2
    return temp + dtdp(mid, (p0 + p1) / 2) * (p1 - p0)


def ascend(env: Environment, height: float, z0: float, temp: float, q: float, mix: float, count_from: Optional[float] = None) -> Ascent:
    """Lifts a parcel from z0 (m) with temperature temp (C) and mixing ratio q (sounding.ts:29-68)."""
    if count_from is None:
        count_from = z0
    dz = 25.0
    saturated, lcl, lfc, el, cape, cin = False, None, None, None, 0.0, 0.0
    area, rising = 0.0, False
    z = z0
    while z <= height:
        sat = env.qsat(temp, z)
        if q >= sat:
            saturated = True
            q = sat
            if lcl is None:
                lcl = z / 1000
        tv = (temp + 273.15) * (1 + .61 * q)
        env_t = env.temperature_env(z)
        env_tv = (env_t + 273.15) * (1 + .61 * env.q_env(z))
        b = G * (tv - env_tv) / env_tv
        if z >= count_from:
            if z - dz < count_from and count_from > z0:
                if b < 0:
                    cin += -b * (z - z0) / 2
                elif lcl is not None:
                    cape += b * (z - z0) / 2
            if lcl is not None and lfc is None and b > 0:
                lfc = z / 1000
                rising = True
            if lfc is None:
                cin -= b * dz
            if lfc is not None:
                area += b * dz
                if b > 0:
                    rising = True
                elif rising and z / 1000 > lfc + .2:
                    rising = False
                    el = z / 1000
                    cape = area - b * dz
        p0, p1 = env.pressure_at(z), env.pressure_at(z + dz)
        temp = moist_step(env, temp, p0, p1) if saturated else (temp + 273.15) * (p1 / p0) ** KAPPA - 273.15
        temp = lerp(temp, env.temperature_env(z + dz), mix)
        q = lerp(q, env.q_env(z + dz), mix)
        z += dz
    if rising:
        el = None
        cape = area
    return Ascent(max(0.0, cape), max(0.0, cin), lcl, lfc, el)


def height_of(env: Environment, p: float, top: float) -> float:
    """Height (m) where the environment's pressure falls to p, 10 m resolution (sounding.ts:94)."""
    z = 0.0
    while z < top and env.pressure_at(z) > p:
        z += 10
    return z


def theta_e(t: float, q: float, p: float) -> float:
    """Equivalent potential temperature (Bolton 1980), K (sounding.ts:97-100)."""
    tk = t + 273.15
    e = max(1e-3, q * p / (EPS + q)) / 100
    tl = 2840 / (3.5 * math.log(tk) - math.log(e) - 4.805) + 55
    r = q * 1000
    return tk * (100000 / p) ** (.2854 * (1 - .00028 * r)) * math.exp((3.376 / tl - .00254) * r * (1 + .00081 * r))


def lift_parcel(env: Environment, height: float, kind: str) -> Ascent:
    """A standard parcel, no excess and no entrainment: 'sb' surface, 'ml' mixed layer over the lowest 100 hPa, 'mu'
    the highest theta-e in the lowest 300 hPa (sounding.ts:121-136)."""
    p0 = env.pressure_at(0)
    if kind == "ml":
        ml_top = height_of(env, p0 - 10000, height)
        th, qs, w = 0.0, 0.0, 0.0
        z = 0.0
        while z < ml_top:
            dp = env.pressure_at(z) - env.pressure_at(z + 10)
            th += env.theta_env(z + 5) * dp
            qs += env.q_env(z + 5) * dp
            w += dp
            z += 10
        a = ascend(env, height, 0.0, th / w * (p0 / 100000) ** KAPPA - 273.15, qs / w, 0.0, ml_top)
        return a
    z0 = 0.0
    if kind == "mu":
        mu_top = height_of(env, p0 - 30000, height)
        best = -math.inf
        z = 0.0
        while z <= mu_top:
            te = theta_e(env.temperature_env(z), env.q_env(z), env.pressure_at(z))
            if te > best:
                best, z0 = te, z
            z += 25
    a = ascend(env, height, z0, env.temperature_env(z0), env.q_env(z0), 0.0)
    a.start = z0 / 1000
    return a


def parcel_indices(env: Environment, height: float) -> dict:
    """The surface-based, mixed-layer and most-unstable parcels (sounding.ts:139-160, without the downdraft CAPE)."""
    return {k: lift_parcel(env, height, k) for k in ("sb", "ml", "mu")}
