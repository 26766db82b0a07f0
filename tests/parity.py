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
