"""Admission by HBM budget (GPU): a context whose budget holds exactly two standard runs refuses a third with
SG_ERR_BUDGET and a message, reuses a retired run's memory, and a serving loop with that budget keeps a third
request queued until a retirement frees memory; that request's result is bitwise the one it gets alone."""
import numpy as np
import pytest

from meteolab_gb300.grid import DEFAULT_GRID, create_grid
from meteolab_gb300.scenarios import CARRIED, baseline_run

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300 import runtime
    return runtime


def test_a_third_run_beyond_the_budget_is_refused(lib):
    spec = baseline_run(create_grid(DEFAULT_GRID), seed=42)
    nb = lib.run_bytes(spec.grid)
    assert nb > 0
    c = lib.Context(0, hbm_budget=2 * nb)
    a, b = c.create(spec), c.create(spec)
    with pytest.raises(lib.StormGpuError, match="beyond the HBM budget") as e:
        c.create(spec)
    assert e.value.code == 2
    a.retire()
    d = c.create(spec)      # the retired run's allocation comes back from the pool
    d.step(1)
    assert d.status()["steps"] == 1
    for r in (b, d):
        r.retire()
    c.close()


def test_server_waits_for_a_retirement_when_the_budget_is_full(lib):
    specs = [baseline_run(create_grid(DEFAULT_GRID), seed=s) for s in (21, 22, 23)]
    steps = [3, 6, 4]
    alone = lib.Context(0)
    ref = []
    for s, n in zip(specs, steps):
        r = alone.create(s)
        r.step(n)
        ref.append(r.read())
        r.retire()
    alone.close()

    c = lib.Context(0, hbm_budget=2 * lib.run_bytes(specs[0].grid))
    srv = lib.Server(c, max_active=8)          # slots are not the limit here: memory is
    for tag, (s, n) in enumerate(zip(specs, steps)):
        srv.submit(s, n, tag)
    got, log = {}, []
    for _ in range(40):
        done, active, queued = srv.iterate()
        log.append((active, queued, list(done)))
        for tag in done:
            got[tag] = srv.collect(tag, specs[tag].grid.n)
        if len(got) == 3:
            break
    srv.close()
    c.close()
    # two admitted, the third queued behind the budget until the first (3 steps) finished and was collected
    assert log[0][:2] == (2, 1), log
    first_done = next(k for k, e in enumerate(log) if e[2])
    assert all(e[1] == 1 for e in log[:first_done + 1]), log
    assert log[first_done + 1][1] == 0, log
    assert sorted(got) == [0, 1, 2]
    for tag in range(3):
        for k in CARRIED:
            assert np.array_equal(got[tag][k], ref[tag][k]), (tag, k)
