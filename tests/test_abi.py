"""The C ABI library: it builds for sm_103a here, loads without a GPU, and exports every function include/stormgpu.h
declares; the Python host mirror binds each of them. No compute call is made (no GPU on this machine)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "stormgpu.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(sg_\w+)\s*\(", src, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    from meteolab_gb300 import build
    build.build()
    return ctypes.CDLL(os.path.join(ROOT, "meteolab_gb300", "libstormgpu.so"))


def test_header_declares_the_entry_points():
    names = declared()
    for must in ("sg_context_create", "sg_run_create", "sg_run_step", "sg_batch_step", "sg_run_read_fields",
                 "sg_run_write_fields", "sg_run_read_columns", "sg_run_status", "sg_run_retire", "sg_last_error",
                 "sg_context_destroy", "sg_server_submit", "sg_server_iterate", "sg_server_collect"):
        assert must in names


def test_library_exports_every_declared_function(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_binds_every_declared_function(lib):
    from meteolab_gb300 import runtime
    src = open(runtime.__file__).read()
    unbound = [n for n in declared() if n not in src]
    assert not unbound, unbound


def test_context_create_fails_cleanly_without_a_device(lib):
    lib.sg_context_create.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]
    h = ctypes.c_void_p()
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is visible")
    assert lib.sg_context_create(0, 0, ctypes.byref(h)) != 0
    assert not h.value


def test_napi_addon_compiles_against_the_documented_api():
    """The N-API addon (meteolab_gb300/csrc/napi/stormgpu_napi.c) compiles without a warning against declarations of
    the Node-API calls it makes (tests/napi_stub/node_api.h; no Node here to provide its own header)."""
    import shutil
    import subprocess
    cc = shutil.which("cc") or shutil.which("gcc")
    if not cc:
        pytest.skip("no C compiler")
    src = os.path.join(ROOT, "meteolab_gb300", "csrc", "napi", "stormgpu_napi.c")
    r = subprocess.run([cc, "-std=c11", "-fsyntax-only", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
                        "-I", os.path.join(ROOT, "tests", "napi_stub"), src], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_static_check_refuses_short_level_arrays():
    """The Python mirror of sg_divergence_max_static checks the level arrays' lengths before the C side reads them."""
    from meteolab_gb300.grid import DEFAULT_GRID, create_grid
    from meteolab_gb300.runtime import divergence_max_static
    g = create_grid(DEFAULT_GRID)
    with pytest.raises(ValueError, match="levels"):
        divergence_max_static(0, 0, 0, 0, g, [1.0] * (g.nz - 1))


def test_run_bytes_grow_with_the_extra_fields(lib):
    """What admission by budget counts (sg_run_bytes_for, host arithmetic only): the extra field sets and fall speeds
    of a two-moment run, twice the fall speeds with two-moment graupel and hail, the lightning's buffers on top; the
    graupel and hail moments need two-moment rain and the ice microphysics (ice2m(), src/core/model.ts:914)."""
    from meteolab_gb300 import runtime
    from meteolab_gb300.grid import DEFAULT_GRID, create_grid
    from meteolab_gb300.scenarios import Switches
    g = create_grid(DEFAULT_GRID)
    plain, rain2, ice2 = (runtime.run_bytes(g, Switches(rain_moments=r, ice_moments=i)) for r, i in ((1, 1), (2, 1), (2, 2)))
    elec_ice2 = runtime.run_bytes(g, Switches(rain_moments=2, ice_moments=2, lightning=1))
    assert plain == runtime.run_bytes(g) < rain2 < ice2 < elec_ice2
    assert ice2 - rain2 >= 6 * g.n * 4  # graupel's and hail's three speeds each
    assert runtime.run_bytes(g, Switches(rain_moments=1, ice_moments=2)) == plain
    assert runtime.run_bytes(g, Switches(rain_moments=2, ice_moments=2, ice=0)) == rain2
