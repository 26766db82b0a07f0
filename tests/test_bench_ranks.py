"""The multi-rank logic of bench.py (replicas only) on the CPU: two gloo ranks, as torchrun launches them."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    from meteolab_gb300.grid import DEFAULT_GRID, create_grid

    class A:
        gpus = world
    r, w, local, pg = bench.dist_setup(A)
    assert (r, w, local) == (rank, world, rank) and pg is not None
    bench.barrier(pg)
    ms = bench.allmax(pg, 10.0 + rank)  # the slower rank sets the job's time
    grid = create_grid(DEFAULT_GRID)
    members = bench.rank_members(grid, 2, rank)
    out.put((rank, ms, bench.job_value(grid.n * 2, w, 5, ms), [m.seed for m in members]))
    pg.destroy_process_group()


def test_two_ranks_take_the_max_time_and_own_seeds():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, ms0, v0, seeds0), (r1, ms1, v1, seeds1) = got
    assert ms0 == ms1 == 11.0
    assert v0 == v1 == 64000 * 2 * 2 * 5 / 11e-3
    assert not set(seeds0) & set(seeds1)  # independent replicas


def test_reference_arm_prints_on_rank_zero_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        gpus, steps, warmup, members = 2, 1, 0, 64
    bench.reference_arm(A, 1, None)
    assert capsys.readouterr().out == ""


def test_clock_summary_reads_the_reason_bits_and_the_timed_samples():
    """The clock record of the timed region: NVML samples (SM MHz, clock-event reason bits) give the median and the
    reasons that were active at any sample; nvidia-smi lines count only from the region's start."""
    sys.path.insert(0, ROOT)
    import bench
    c = bench.Clocks(0)
    c.nvml, c.max_mhz = ("lib", None, None), 2070.0
    c.samples = [(2070.0, 0), (2070.0, 0x4), (1980.0, 0x4 | 0x1), (2070.0, 0)]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["reasons"] == ["sw_power_cap"] and s["samples"] == 4
    c.samples.append((1500.0, 0x40))
    assert bench.Clocks.summary(c)["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    smi = bench.Clocks(0)
    smi.lines = ["0, 1200, 2070, 300, Not Active, Not Active, Not Active, Not Active, Not Active",
                 "0, 2070, 2070, 900, Active, Not Active, Not Active, Not Active, Active",
                 "0, 2065, 2070, 950, Not Active, Not Active, Not Active, Not Active, Not Active"]
    smi.first = 1  # the idle sample before the region is left out
    s = smi.summary()
    assert s["samples"] == 2 and s["sm_mhz"] == (2070 + 2065) / 2 and s["reasons"] == ["sw_power_cap"]
