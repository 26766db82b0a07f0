"""sg_divergence_max_static, the divergence check that allocates nothing, against the entry point it mirrors
(sg_run_divergence). Collected last: it must pass alone and after every other test in the same process."""
import numpy as np
import pytest

from meteolab_gb300.grid import DEFAULT_GRID, GridOptions, create_grid
from meteolab_gb300.scenarios import baseline_run

pytestmark = pytest.mark.gpu


def test_static_scratch_divergence_matches_the_run_entry_point():
    torch = pytest.importorskip("torch")
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import Context, StormGpuError, divergence_max_static
    ctx = Context(0)
    spec = baseline_run(create_grid(DEFAULT_GRID), seed=42)
    r = ctx.create(spec)
    r.step(5)
    ref = r.divergence()
    f = r.read(("u", "v", "w"))
    dev = {k: torch.from_numpy(f[k]).to("cuda:0") for k in f}
    torch.cuda.synchronize()
    args = (dev["u"].data_ptr(), dev["v"].data_ptr(), dev["w"].data_ptr(), spec.grid, spec.env.rho)
    first = divergence_max_static(0, *args)
    second = divergence_max_static(0, *args)  # two calls in a row: the scratch is cleared each time
    assert first == ref and second == ref, (first, second, ref)
    assert ref > 0.0

    # new data: the next call reports the new maximum, not the one left in the scratch
    w2 = f["w"] * np.float32(0.25)
    r.write({"w": w2})
    ref2 = r.divergence()
    dev["w"].copy_(torch.from_numpy(w2))
    torch.cuda.synchronize()
    third = divergence_max_static(0, *args)
    assert third == ref2 and ref2 != ref

    # a NaN in the velocities: a non-finite maximum and SG_ERR_NONFINITE, not a finite number that passes a check
    dev["w"][777] = float("nan")
    torch.cuda.synchronize()
    with pytest.raises(StormGpuError, match="non-finite") as e:
        divergence_max_static(0, *args)
    assert e.value.code == 5
    assert torch.cuda.current_device() == 0
    dev["w"].copy_(torch.from_numpy(w2))
    torch.cuda.synchronize()
    assert divergence_max_static(0, *args) == ref2  # the scratch holds no NaN into the next call

    # beyond the static level table: rejected with a message
    tall = create_grid(GridOptions(8, 8, 200, 9600.0, 9000.0, 18900.0, 50.0))
    with pytest.raises(StormGpuError, match="static level table"):
        divergence_max_static(0, *args[:3], tall, np.ones(200))
    r.retire()
    ctx.close()
