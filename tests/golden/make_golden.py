"""Generates tests/golden/step_small.npz: golden output of the StormLab step on a small grid.

The reference (TypeScript) cannot run here or on the GPU machine, so the vectors come from the oracle in pure FP64 mode
(oracle/, the reference step restated in C++ and pinned by the reference's known-answer tests, tests/test_oracle_kat.py).
They pin the host-side set-up (grid, sounding, initial state: a SHA-256 of the initial fields) and the oracle itself
against regressions, and give the device step a fixed target that needs no oracle at run time.

Run from the repository root: python tests/golden/make_golden.py
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle")]

from meteolab_gb300.grid import GridOptions, create_grid  # noqa: E402
from meteolab_gb300.scenarios import CARRIED, baseline_run  # noqa: E402

# 12 x 10 x 16 nodes at the standard spacing (dx 1.2 km, dy 1.125 km), 100 m at the ground to 18.9 km, a 3 K bubble
# in a 16 g/kg sounding
# and +-0.1 K noise (seed 7). Snapshots: after SPIN steps of 3 s (the developed state, with cloud and rain) and after
# SPIN + STEPS (continued from the snapshot rounded to FP32, so the second snapshot follows from the stored first).
GRID = GridOptions(12, 10, 16, 12 * 1200.0, 10 * 1125.0, 18900.0, 100.0)
SEED, SPIN, STEPS = 7, 420, 2
PATH = os.path.join(HERE, "step_small.npz")


def spec():
    return baseline_run(create_grid(GRID), seed=SEED, bubble=3.0, qv_max=0.016)


def initial_digest(fields) -> str:
    h = hashlib.sha256()
    for k in CARRIED:
        h.update(np.ascontiguousarray(fields[k], dtype=np.float32).tobytes())
    return h.hexdigest()


def main():
    import pyoracle
    s = spec()
    m = pyoracle.OracleModel(s, fp64=True)
    m.step(s.switches.dt, SPIN)
    out = {f"spun_{k}": m.get(k).astype(np.float32) for k in CARRIED}
    out["spun_precipitation"] = m.get("precipitation").astype(np.float32)
    for k in CARRIED:  # continue from exactly the stored FP32 state, as a restart from the snapshot does
        m.set(k, out[f"spun_{k}"])
    m.step(s.switches.dt, STEPS)
    out.update({f"final_{k}": m.get(k).astype(np.float32) for k in CARRIED})
    out["final_precipitation"] = m.get("precipitation").astype(np.float32)
    out["initial_sha256"] = np.array(initial_digest(s.fields))
    out["spin"] = np.array(SPIN)
    out["steps"] = np.array(STEPS)
    np.savez_compressed(PATH, **out)
    print(f"wrote {PATH} ({os.path.getsize(PATH)} bytes)")


if __name__ == "__main__":
    main()
