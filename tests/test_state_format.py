"""The saved-state format (.meteolab files, src/core/state.ts) on the CPU: the library's readState checks
(sg_state_parse, no device involved) against the format's oracle (oracle/state_format.py) on the reference's own
cases (src/core/state.test.ts:41-68) and on damaged images."""
import json
import struct

import numpy as np
import pytest

import state_format as SF


@pytest.fixture(scope="module")
def parse():
    from meteolab_gb300 import build
    build.build()
    from meteolab_gb300.runtime import StormGpuError, parse_state

    def run(image):
        try:
            return parse_state(image), None
        except StormGpuError as e:
            return None, str(e).split(": ", 1)[1]
    return run


def oracle(image):
    try:
        h, _, _ = SF.read_state(image)
        return h, None
    except SF.StateError as e:
        return None, str(e)


def image(version=5, nx=16, ny=12, nz=50, time=600.0, persisted=30.0, seed=0, config=None):
    rng = np.random.default_rng(seed)
    n, layer = nx * ny * nz, nx * ny
    fields = {k: rng.standard_normal(n).astype(np.float32) for k in SF.fields_of(version)}
    cols = {k: rng.random(layer).astype(np.float32) for k in SF.STATE_COLUMNS}
    cfg = config if config is not None else {"seed": 7, "surfaceTemp": 30.5, "sounding": None, "nested": {"version": 9, "nx": -1}}
    return SF.save_state(fields, cols, cfg, time, persisted, nx, ny, nz, version=version), fields, cols


@pytest.mark.parametrize("version", [1, 2, 3, 4, 5])
def test_every_version_reads_as_the_oracle_reads_it(parse, version):
    img, fields, cols = image(version=version)
    got, err = parse(img)
    ref, rerr = oracle(img)
    assert err is None and rerr is None
    assert (got["version"], got["nx"], got["ny"], got["nz"]) == (version, 16, 12, 50)
    assert got["time"] == ref["time"] == 600.0 and got["persisted"] == ref["persisted"] == 30.0
    assert got["nfields"] == len(SF.fields_of(version))
    # the data start at the 4-byte boundary after the header: the first field's first value is there
    first = np.frombuffer(img, np.float32, count=1, offset=got["data_offset"])[0]
    assert first == fields[SF.STATE_FIELDS[0]][0]


def test_a_version_1_file_as_the_reference_builds_it(parse):
    # state.test.ts:41-46: header by hand, 12 fields and 3 columns, every value 1
    nx, ny, nz = 16, 12, 50
    n, layer = nx * ny * nz, nx * ny
    js = json.dumps({"format": "meteolab-state", "version": 1, "config": {}, "time": 60, "persisted": 0, "nx": nx, "ny": ny, "nz": nz}).encode()
    start = -(-(8 + len(js)) // 4) * 4
    img = b"MLAB" + struct.pack("<I", len(js)) + js + b"\0" * (start - 8 - len(js)) + np.ones(12 * n + 3 * layer, np.float32).tobytes()
    got, err = parse(img)
    assert err is None and got["version"] == 1 and got["time"] == 60 and got["nfields"] == 12
    h, fields, cols = SF.read_state(img)
    assert fields["hail"][0] == 1 and "iceNumber" not in fields


def damaged():
    good, _, _ = image()
    length = struct.unpack("<I", good[4:8])[0]
    header = json.loads(good[8:8 + length])

    def with_header(h, extra_bytes=0):
        js = json.dumps(h).encode()
        start = -(-(8 + len(js)) // 4) * 4
        body = good[-(len(good) - (-(-(8 + length) // 4) * 4)):]
        return b"MLAB" + struct.pack("<I", len(js)) + js + b"\0" * (start - 8 - len(js)) + body + b"\0" * extra_bytes

    cases = {
        "not a state file": "hello world, not a state".encode(),
        "too short": b"MLA",
        "wrong magic": b"MLAX" + good[4:],
        "cut by 4 bytes": good[:-4],
        "one byte more": good + b"\0",
        "header past the end": good[:4] + struct.pack("<I", len(good)) + good[8:],
        "header not JSON": good[:8] + b"{" * length + good[8 + length:],
        "header trailing text": with_header(header)[:8] + b"x" + with_header(header)[9:],
        "format missing": with_header({k: v for k, v in header.items() if k != "format"}),
        "format wrong": with_header({**header, "format": "other"}),
        "version 6": with_header({**header, "version": 6}),
        "version as text": with_header({**header, "version": "5"}),
        "time negative": with_header({**header, "time": -1}),
        "nz missing": with_header({k: v for k, v in header.items() if k != "nz"}),
        "nx as text": with_header({**header, "nx": "16"}),
        "header is a list": b"MLAB" + struct.pack("<I", 2) + b"[]" + b"\0\0" + good[-(len(good) - (-(-(8 + length) // 4) * 4)):],
        "grid of another size": with_header({**header, "nx": 17}),
    }
    return cases


@pytest.mark.parametrize("name", list(damaged().keys()))
def test_damaged_images_are_refused_with_the_reference_messages(parse, name):
    img = damaged()[name]
    got, err = parse(img)
    ref, rerr = oracle(img)
    assert got is None and ref is None, name
    assert err == rerr, (name, err, rerr)


def test_refusal_messages_are_the_reference_ones(parse):
    # state.test.ts:62-64: not a state file; an image cut by 4 bytes is a size mismatch
    assert parse("hello world, not a state".encode())[1] == "this is not a MeteoLab state file"
    good, _, _ = image()
    assert parse(good[:-4])[1] == "the file's size does not match the grid"
