"""TEST INFRASTRUCTURE ONLY — the oracle of the saved-state format: a plain-Python restatement of the reference's
.meteolab files (src/core/state.ts), used by tests/ to write images the device loads and to read the images the device
saves. Imported by tests/ only; never by the product.

Layout (state.ts:1-4, :43-53): b'MLAB', the JSON header's length as uint32 little endian, the JSON header, zero
padding to a multiple of 4 bytes, then float32 fields in STATE_FIELDS order (n = nx*ny*nz each) and the ground
columns in STATE_COLUMNS order (nx*ny each).
"""
from __future__ import annotations

import json
import math
import struct
from typing import Dict, Optional

import numpy as np

# state.ts:9-10
STATE_FIELDS = ("u", "v", "w", "theta", "q", "cloud", "rain", "cold", "ice", "snow", "graupel", "hail", "chargeIce",
                "chargeGraupel", "chargeRain", "chargeAir", "iceNumber", "rainNumber", "graupelNumber", "graupelVolume",
                "hailNumber", "hailVolume")
STATE_COLUMNS = ("precipitation", "hailGround", "hailSize")
MAGIC, VERSION = b"MLAB", 5   # state.ts:18


def fields_of(version: int):
    """state.ts:32: the fields a file of this version holds."""
    count = {1: 12, 2: 16, 3: 17, 4: 18}.get(version, len(STATE_FIELDS))
    return STATE_FIELDS[:count]


class StateError(ValueError):
    pass


def save_state(fields: Dict[str, np.ndarray], columns: Dict[str, np.ndarray], config, time: float, persisted: float,
               nx: int, ny: int, nz: int, version: int = VERSION, header: Optional[dict] = None) -> bytes:
    """saveState (state.ts:43-53); `version` < 5 writes an older file (its field list), as the reference's tests build
    them by hand (state.test.ts:42-46). Fields absent from `fields` are written as zeros."""
    h = header if header is not None else {"format": "meteolab-state", "version": version, "config": config, "time": time,
                                           "persisted": persisted, "nx": nx, "ny": ny, "nz": nz}
    js = json.dumps(h, separators=(",", ":")).encode()
    start = math.ceil((8 + len(js)) / 4) * 4
    n, layer = nx * ny * nz, nx * ny
    parts = [MAGIC, struct.pack("<I", len(js)), js, b"\0" * (start - 8 - len(js))]
    for k in fields_of(version):
        a = fields.get(k)
        parts.append((np.zeros(n, np.float32) if a is None else np.asarray(a, np.float32).ravel()).tobytes())
    for k in STATE_COLUMNS:
        a = columns.get(k)
        parts.append((np.zeros(layer, np.float32) if a is None else np.asarray(a, np.float32).ravel()).tobytes())
    return b"".join(parts)


def read_state(buf: bytes):
    """readState (state.ts:55-68): (header, {field: array}, {column: array}); StateError with the reference's message."""
    if len(buf) < 8 or buf[:4] != MAGIC:
        raise StateError("this is not a MeteoLab state file")
    length = struct.unpack("<I", buf[4:8])[0]
    if 8 + length > len(buf):
        raise StateError("the file is truncated")
    try:
        header = json.loads(buf[8:8 + length].decode("utf-8", errors="replace"))
    except ValueError:
        raise StateError("the file's header is damaged")
    version = header.get("version") if isinstance(header, dict) else None
    fmt = header.get("format") if isinstance(header, dict) else None
    if fmt != "meteolab-state" or isinstance(version, bool) or version not in (1, 2, 3, 4, 5):
        raise StateError("unknown file format or version")
    for k in ("time", "persisted", "nx", "ny", "nz"):
        v = header.get(k)
        if isinstance(v, bool) or not isinstance(v, (int, float)) or not math.isfinite(v) or v < 0:
            raise StateError("the file's header is damaged")
    start = math.ceil((8 + length) / 4) * 4
    cells = header["nx"] * header["ny"]
    names = fields_of(version)
    size = len(names) * cells * header["nz"] + len(STATE_COLUMNS) * cells
    if len(buf) != start + size * 4:
        raise StateError("the file's size does not match the grid")
    data = np.frombuffer(buf, np.float32, count=int(size), offset=start)
    n = int(cells * header["nz"])
    fields = {k: data[j * n:(j + 1) * n].copy() for j, k in enumerate(names)}
    o = len(names) * n
    columns = {k: data[o + j * int(cells):o + (j + 1) * int(cells)].copy() for j, k in enumerate(STATE_COLUMNS)}
    return header, fields, columns
