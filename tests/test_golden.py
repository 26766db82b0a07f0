"""The oracle against the committed golden vectors (tests/golden/step_small.npz, made by tests/golden/make_golden.py):
pins the host-side set-up (grid, sounding, initial state) and the oracle's step against regressions."""
import importlib.util
import os

import numpy as np
import pytest

import pyoracle as O
from parity import FLOOR, rel_l2
from meteolab_gb300.scenarios import CARRIED

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def golden():
    s = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(s)
    s.loader.exec_module(mg)
    return mg, np.load(os.path.join(HERE, "golden", "step_small.npz"))


def test_initial_state_matches_golden(golden):
    mg, d = golden
    assert mg.initial_digest(mg.spec().fields) == str(d["initial_sha256"])


def test_fp64_oracle_reproduces_golden_run(golden):
    mg, d = golden
    spec = mg.spec()
    m = O.OracleModel(spec, fp64=True)
    m.step(spec.switches.dt, int(d["spin"]))
    for k in CARRIED:
        assert rel_l2(m.get(k).astype(np.float32), d[f"spun_{k}"], FLOOR.get(k, 0.0)) < 1e-6, k
        m.set(k, m.get(k).astype(np.float32))
    m.step(spec.switches.dt, int(d["steps"]))
    for k in CARRIED:
        assert rel_l2(m.get(k).astype(np.float32), d[f"final_{k}"], FLOOR.get(k, 0.0)) < 1e-6, k


def test_oracle_restarts_from_golden_snapshot(golden):
    """Stepping from the stored (FP32) developed state lands on the stored result: the restart path the device test
    takes."""
    mg, d = golden
    spec = mg.spec()
    m = O.OracleModel(spec, fp64=True)
    for k in CARRIED:
        m.set(k, d[f"spun_{k}"])
    m.step(spec.switches.dt, int(d["steps"]))
    for k in CARRIED:
        assert rel_l2(m.get(k).astype(np.float32), d[f"final_{k}"], FLOOR.get(k, 0.0)) < 1e-6, k
