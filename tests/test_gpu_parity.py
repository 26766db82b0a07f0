"""Parity of the device step with the oracle, through the C ABI (GPU).

Tolerances: the device computes the fields and all stencil arithmetic in FP32 (FP64 only in the tridiagonal
solves and the budget sums); the oracle is the reference's algorithm in FP64 arithmetic. Per field after one step
the relative L2 error is held to 1e-5 (with the absolute floors of tests/parity.py for fields that are near zero);
stage by stage within a step (FP64 oracle) to 1e-5; over 100 steps of a growing storm to 1e-4 (measured 2.1e-5: FP32
rounding amplified by the convective instability the storm grows from).
"""
import numpy as np
import pytest

import pyoracle as O
from parity import FLOOR, developed_state, dual_divergence, field_errors, pressure_gradient, rel_l2, threads
from meteolab_gb300.grid import DEFAULT_GRID, LARGE_GRID, GridOptions, create_grid
from meteolab_gb300.scenarios import CARRIED, baseline_run

pytestmark = pytest.mark.gpu
DT = 3.0


@pytest.fixture(scope="module")
def ctx():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import Context
    c = Context()
    yield c
    c.close()


@pytest.fixture(scope="module")
def storm():
    """A developed storm on the standard grid: 300 oracle steps (15 min) from the benchmark initial state."""
    spec = baseline_run(create_grid(DEFAULT_GRID), seed=42)
    return developed_state(spec, 300)


def _report(title, errs):
    print(f"\n{title}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))


def test_step_parts_match_oracle(ctx, storm):
    """Part by part within one step (beginStep, dynamics, physicsStep, mixStep, final projection), against the FP64
    oracle run through the same parts."""
    o = O.OracleModel(storm, fp64=True, threads=threads())
    r = ctx.create(storm)
    thb = np.repeat(storm.env.theta, storm.grid.layer)
    # where each field lives on the device after each part (set index)
    where = {1: {k: 0 for k in CARRIED}, 2: {k: 1 for k in CARRIED},
             3: {k: (0 if k in ("rain", "snow", "graupel", "hail", "cold") else 2) for k in CARRIED},
             4: {k: 0 for k in CARRIED}, 5: {k: 0 for k in CARRIED}}
    worst = {}
    for part in (1, 2, 3, 4, 5):
        o.step_part(DT, part)
        r.debug_part(part)
        got = {k: r.debug_read_set(where[part][k], k) for k in CARRIED}
        thp = got["theta"].astype(np.float64)
        got["theta"] = thp + thb
        ref = o.fields()
        errs = field_errors(got, ref)
        errs["theta'"] = rel_l2(thp, ref["theta"] - thb, FLOOR["theta'"])
        _report(f"part {part}", errs)
        worst[part] = errs
    for part, errs in worst.items():
        bad = {k: v for k, v in errs.items() if v > 1e-5}
        assert not bad, f"part {part}: {bad}"
    r.retire()


def test_one_step_against_fp64_oracle(ctx, storm):
    """Every field within 1e-5 relative L2 of the FP64 oracle after one step (from the developed storm)."""
    o64 = O.OracleModel(storm, fp64=True, threads=threads())
    o64.step(DT, 1)
    ref = o64.fields()
    r = ctx.create(storm)
    r.step(1)
    got = r.read()
    errs = field_errors(got, ref)
    thb = np.repeat(storm.env.theta, storm.grid.layer)
    # the device's own departure (the ABI hands back the full theta rounded to FP32, as the reference stores it)
    errs["theta'"] = rel_l2(r.debug_read_set(0, "theta"), ref["theta"] - thb, FLOOR["theta'"])
    _report("one step vs FP64", errs)
    col = r.columns()
    errs_c = {"precipitation": rel_l2(col["precipitation"], o64.get("precipitation"), 1e-9)}
    _report("columns", errs_c)
    assert max(errs.values()) <= 1e-5, errs
    assert errs_c["precipitation"] <= 1e-5
    r.retire()


def test_hundred_steps_from_rest(ctx):
    """100 steps from the initial state on the standard grid against the FP64 oracle."""
    spec = baseline_run(create_grid(DEFAULT_GRID), seed=7)
    o64 = O.OracleModel(spec, fp64=True, threads=threads())
    o64.step(DT, 100)
    r = ctx.create(spec)
    r.step(100)
    got, ref = r.read(), o64.fields()
    errs = field_errors(got, ref)
    thb = np.repeat(spec.env.theta, spec.grid.layer)
    errs["theta'"] = rel_l2(r.debug_read_set(0, "theta"), ref["theta"] - thb, FLOOR["theta'"])
    _report("100 steps vs FP64", errs)
    st = r.status()
    assert st["steps"] == 100 and st["clipped"] == 0 and not st["failed"]
    assert max(errs.values()) <= 1e-4, errs
    r.retire()


def test_projection_leaves_no_divergence(ctx, storm):
    """The final projection removes the divergence the physics and mixing made. Two measures, both max |D R u| over
    all dual cells relative to the same before the projection: after rounding (the stored FP32 velocities, FP64 on the
    device; FP32 rounding of u bounds it) and before rounding (u - dt G p formed in FP64 from the FP32 velocities and
    the FP32 pressure the solve returned: the accuracy of the solve itself)."""
    r = ctx.create(storm)
    for part in (1, 2, 3, 4):
        r.debug_part(part)
    before = r.divergence()
    pre = r.read(("u", "v", "w"))
    r.debug_part(5)
    after = r.divergence()
    g = storm.grid
    gx, gy, gz = pressure_gradient(r.pressure(), g)
    dt = storm.switches.dt
    u = pre["u"].astype(np.float64) - dt * gx
    v = pre["v"].astype(np.float64) - dt * gy
    w = pre["w"].astype(np.float64) - dt * gz
    exact = float(np.max(np.abs(dual_divergence(u, v, w, g, storm.env.rho))))
    ref = float(np.max(np.abs(dual_divergence(pre["u"], pre["v"], pre["w"], g, storm.env.rho))))
    print(f"\nmax |D R u|: before the final projection {before:.3e}, after {after:.3e} (ratio {after / before:.2e} after "
          f"rounding), {exact / ref:.2e} before rounding")
    assert after < 1e-4 * before
    assert exact <= 1e-8 * ref  # the refined projection (Switches.refine_projection, on by default)
    r.retire()


def test_runs_are_deterministic_and_batch_independent(ctx, storm):
    """A run alone and the same run inside an uneven batch (standard + large) give bitwise equal fields."""
    alone = ctx.create(storm)
    alone.step(3)
    a = alone.read()
    big = baseline_run(create_grid(LARGE_GRID), seed=5)
    x, y = ctx.create(storm), ctx.create(big)
    ctx.batch_step([x, y], 3)
    b = x.read()
    for k in CARRIED:
        assert np.array_equal(a[k], b[k]), k
    z = ctx.create(big)
    z.step(3)
    c, d = y.read(), z.read()
    for k in CARRIED:
        assert np.array_equal(c[k], d[k]), k
    for run in (alone, x, y, z):
        run.retire()


def test_graph_branches_match_the_serial_order(ctx, storm):
    """The captured step runs independent chains on parallel branches (sedimentation beside the face projection, the
    WENO transport of the three stages beside the dynamics transport and the stage projections); launched eagerly the
    same kernels run one after another on one stream. Both orders give bitwise equal fields, for a batch of runs."""
    specs = [storm, baseline_run(create_grid(DEFAULT_GRID), seed=11), baseline_run(create_grid(LARGE_GRID), seed=12)]
    serial = [ctx.create(s) for s in specs]
    ctx.time_steps(serial, 3, graph=False)
    branched = [ctx.create(s) for s in specs]
    ctx.time_steps(branched, 3, graph=True)
    for a, b in zip(serial, branched):
        x, y = a.read(), b.read()
        for k in CARRIED:
            assert np.array_equal(x[k], y[k]), k
    for r in serial + branched:
        r.retire()


def test_row_transform_path_matches_fp64_oracle(storm, monkeypatch):
    """The row-transform path of the spectral solves (x-transforms of row blocks, y-transforms inside the mode
    kernel; what grids too wide for the whole-layer path take, e.g. 320x256) forced on the standard grid: one step
    from the developed storm against the FP64 oracle, every field within 1e-5."""
    from meteolab_gb300.runtime import Context
    monkeypatch.setenv("SG_SPECTRAL_ROWS", "1")
    c = Context(0)
    r = c.create(storm)
    r.step(1)
    got = r.read()
    got_thp = r.debug_read_set(0, "theta")
    m = O.OracleModel(storm, fp64=True, threads=threads())
    m.step(storm.switches.dt, 1)
    ref = {k: m.get(k) for k in CARRIED}
    errs = {k: rel_l2(got[k], ref[k], FLOOR.get(k, 0.0)) for k in CARRIED}
    thb = np.repeat(storm.env.theta, storm.grid.layer)
    errs["theta'"] = rel_l2(got_thp, ref["theta"] - thb, FLOOR["theta'"])
    print("row path:", ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
    bad = {k: v for k, v in errs.items() if not v <= 1e-5}
    r.retire()
    c.close()
    assert not bad, bad


@pytest.mark.parametrize("shape", [(40, 8, 3), (40, 8, 1), (32, 8, 3), (16, 16, 1), (8, 8, 3), (40, 4, 1)])
def test_transport_tiles_give_the_same_bits(ctx, storm, shape):
    """Every transport tile shape and WENO grouping (faces computed alone or as packed pairs) gives bitwise equal
    fields; the autotuner may pick any of them."""
    ctx.set_transport_shape(40, 8, 3)
    ref = ctx.create(storm)
    ref.step(2)
    a = ref.read()
    ctx.set_transport_shape(*shape)
    r = ctx.create(storm)
    r.step(2)
    assert ctx.transport_shape([r])[:3] == shape
    b = r.read()
    ctx.set_transport_shape(0)
    assert ref.status()["failed"] == 0 and r.status()["failed"] == 0
    for k in CARRIED:
        assert np.array_equal(a[k], b[k]), (shape, k)
    ref.retire(); r.retire()


@pytest.mark.parametrize("shape", [(40, 8, 3), (20, 8, 1)])
def test_transport_variants_give_the_same_bits(storm, monkeypatch, shape):
    """The three transport variants give bitwise equal fields, on an uneven batch (standard and large grid) over
    three steps: the tiles whose producer warps move each level's inputs with TMA bulk copies, the per-thread copies
    with two edge warps taking the tile's edge faces, and the per-thread copies with the column threads taking them
    (SG_TRANSPORT_BULK, SG_TRANSPORT_EDGE_WARPS)."""
    from meteolab_gb300.runtime import Context
    specs = [storm, baseline_run(create_grid(LARGE_GRID), seed=14)]
    out = {}
    for bulk, edge in (("1", "1"), ("0", "1"), ("0", "0")):
        monkeypatch.setenv("SG_TRANSPORT_BULK", bulk)
        monkeypatch.setenv("SG_TRANSPORT_EDGE_WARPS", edge)
        c = Context(0)
        c.set_transport_shape(*shape)
        runs = [c.create(s) for s in specs]
        assert c.transport_bulk(runs) == (bulk == "1")
        c.batch_step(runs, 3)
        out[bulk + edge] = [r.read() for r in runs]
        assert all(r.status()["failed"] == 0 for r in runs)
        for r in runs:
            r.retire()
        c.close()
    for variant in ("01", "00"):
        for a, b in zip(out["11"], out[variant]):
            for k in CARRIED:
                assert np.array_equal(a[k], b[k]), (variant, k)


def test_batch_field_io_matches_per_run_calls(ctx, storm):
    runs = [ctx.create(storm), ctx.create(baseline_run(create_grid(LARGE_GRID), seed=8))]
    ctx.batch_step(runs, 2)
    new = []
    for r in runs:
        f = r.read()
        f["u"] = f["u"] + np.float32(1.5)
        f["theta"] = f["theta"] + np.float32(0.25)
        new.append(f)
    ctx.write_fields(runs, new)
    out = [{k: np.empty(r.grid.n, np.float32) for k in CARRIED} for r in runs]
    ctx.read_fields(runs, out)
    for r, f, o in zip(runs, new, out):
        single = r.read()
        for k in CARRIED:
            assert np.array_equal(o[k], single[k]), k
        assert np.array_equal(o["u"], f["u"])
        assert np.max(np.abs(o["theta"] - f["theta"])) < 1e-4  # theta goes through its departure from the base profile
    for r in runs:
        r.retire()


def test_packed_transfer_matches_per_run_calls(ctx, storm):
    runs = [ctx.create(storm), ctx.create(baseline_run(create_grid(LARGE_GRID), seed=9))]
    ctx.batch_step(runs, 2)
    total = sum(r.grid.n for r in runs) * len(CARRIED)
    packed = np.empty(total, np.float32)
    ctx.read_packed(runs, packed)
    o = 0
    for r in runs:
        f = r.read()
        for k in CARRIED:
            assert np.array_equal(packed[o:o + r.grid.n], f[k]), k
            o += r.grid.n
    # write a changed state packed, read it back per run (theta through its departure: FP32-close)
    packed2 = packed.copy()
    packed2[:runs[0].grid.n] += np.float32(1e-4)  # the first run's rain
    ctx.write_packed(runs, packed2)
    back = np.empty_like(packed2)
    ctx.read_packed(runs, back)
    th = [i for i, k in enumerate(CARRIED) if k == "theta"][0]
    o = 0
    for r in runs:
        for j, k in enumerate(CARRIED):
            a, b = back[o:o + r.grid.n], packed2[o:o + r.grid.n]
            if j == th:
                assert np.max(np.abs(a - b)) < 1e-4
            else:
                assert np.array_equal(a, b), k
            o += r.grid.n
    for r in runs:
        r.retire()


@pytest.mark.parametrize("groups,pinned", [(1, False), (3, False), (1, True), (3, True)])
def test_step_with_host_io_matches_separate_calls(ctx, storm, groups, pinned):
    """sg_batch_step_io (write packed, step, read packed; the runs in groups whose copies overlap the other groups'
    steps) gives the bits of the three separate calls, over an uneven batch and two rounds, from pageable and from
    pinned host memory."""
    large = baseline_run(create_grid(LARGE_GRID), seed=11)
    specs = [storm, storm, large, storm, large]
    a = [ctx.create(s) for s in specs]
    b = [ctx.create(s) for s in specs]
    ctx.batch_step(a + b, 3)
    total = sum(r.grid.n for r in a) * len(CARRIED)
    pa = np.empty(total, np.float32)
    ctx.read_packed(a, pa)
    pa[:a[0].grid.n] += np.float32(2e-4)  # a change the host makes between steps (the first run's rain)
    if pinned:
        import torch
        pb = torch.empty(total, dtype=torch.float32, pin_memory=True).numpy()
        pb[:] = pa
    else:
        pb = pa.copy()
    for _ in range(2):
        ctx.write_packed(a, pa)
        ctx.batch_step(a, 1)
        ctx.read_packed(a, pa)
        ctx.batch_step_io(b, pb, steps=1, groups=groups)
        assert np.array_equal(pa, pb)
    for r in a + b:
        r.retire()


@pytest.mark.parametrize("groups", [1, 3])
def test_round_trips_every_step_match_one_call_a_step(ctx, storm, groups):
    """sg_batch_step_round_trips (a round trip through the host buffer every step, the groups pipelined across steps)
    gives the bits of one sg_batch_step_io call a step, over three steps of an uneven batch."""
    large = baseline_run(create_grid(LARGE_GRID), seed=13)
    specs = [storm, large, storm, large, storm]
    a = [ctx.create(s) for s in specs]
    b = [ctx.create(s) for s in specs]
    total = sum(r.grid.n for r in a) * len(CARRIED)
    pa = np.empty(total, np.float32)
    ctx.read_packed(a, pa)
    pb = pa.copy()
    for _ in range(3):
        ctx.batch_step_io(a, pa, steps=1, groups=groups)
    ctx.batch_round_trips(b, pb, steps=3, groups=groups)
    assert np.array_equal(pa, pb)
    for x, y in zip(a, b):
        assert x.status()["steps"] == y.status()["steps"] == 3
    for r in a + b:
        r.retire()


def test_autotuner_picks_a_valid_shape(ctx, storm):
    runs = [ctx.create(storm) for _ in range(4)]
    tx, ty, g, mb = ctx.transport_shape(runs)
    assert tx * ty <= 320 and g in (1, 3) and mb in (2, 3)
    for r in runs:
        r.retire()


@pytest.mark.parametrize("quantum", [1, 3])
def test_serving_gives_the_same_result_alone_and_in_the_mix(ctx, storm, quantum):
    """Requests admitted while others are on the device finish with the fields they get when stepped alone, whether
    an iteration advances one step or several."""
    from meteolab_gb300.runtime import Server
    specs = [storm, baseline_run(create_grid(LARGE_GRID), seed=11), baseline_run(create_grid(DEFAULT_GRID), seed=12)]
    steps = [6, 4, 5]
    ref = []
    for s, n in zip(specs, steps):
        r = ctx.create(s)
        r.step(n)
        ref.append(r.read())
        r.retire()
    srv = Server(ctx, max_active=2)
    srv.set_quantum(quantum)
    srv.submit(specs[0], steps[0], 0)
    srv.submit(specs[1], steps[1], 1)
    got, it = {}, 0
    while len(got) < 3 and it < 50:
        done, active, queued = srv.iterate()
        assert 1 <= srv.last_steps <= quantum or not (active or done)
        for tag in done:
            got[tag] = srv.collect(tag, specs[tag].grid.n)
        if it == 1:
            srv.submit(specs[2], steps[2], 2)  # arrives while two others are stepping; waits for a slot
        it += 1
    srv.close()
    assert sorted(got) == [0, 1, 2]
    for tag in range(3):
        for k in CARRIED:
            assert np.array_equal(got[tag][k], ref[tag][k]), (tag, k)


def test_nonfinite_run_fails_alone(ctx, storm):
    """A NaN put into one run's state marks that run failed; the run batched with it is untouched."""
    bad = {k: v.copy() for k, v in storm.fields.items()}
    bad["theta"][12345] = np.nan
    from meteolab_gb300.scenarios import RunSpec
    sick = ctx.create(RunSpec(storm.grid, storm.env, storm.switches, bad))
    well = ctx.create(storm)
    ctx.batch_step([sick, well], 2)
    assert sick.status()["failed"] == 1
    assert well.status()["failed"] == 0
    ref = ctx.create(storm)
    ref.step(2)
    a, b = well.read(), ref.read()
    for k in CARRIED:
        assert np.array_equal(a[k], b[k]), k
    for r in (sick, well, ref):
        r.retire()


def test_step_with_host_io_refuses_bad_arguments(ctx, storm):
    """sg_batch_step_io: an empty batch, a run named twice and a negative step count are refused with a message; a
    group count out of 1..8 is brought into it."""
    from meteolab_gb300.runtime import StormGpuError
    r = ctx.create(storm)
    buf = np.empty(r.grid.n * len(CARRIED), np.float32)
    ctx.read_packed([r], buf)
    with pytest.raises(StormGpuError, match="empty batch"):
        ctx.batch_step_io([], buf)
    with pytest.raises(StormGpuError, match="twice"):
        ctx.batch_step_io([r, r], np.empty(2 * buf.size, np.float32))
    with pytest.raises(StormGpuError, match="negative step count"):
        ctx.batch_step_io([r], buf, steps=-1)
    before = buf.copy()
    ctx.batch_step_io([r], buf, steps=1, groups=0)
    ctx.batch_step_io([r], buf, steps=0, groups=99)
    assert not np.array_equal(before, buf) and np.all(np.isfinite(buf))
    r.retire()
