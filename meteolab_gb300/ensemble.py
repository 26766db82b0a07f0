"""The ensemble runner over device runs and the series checkpoint, the reference's host logic around the step:
``runMember`` and ``MemberResult`` (src/ensemble/member.ts:13-107) with every member of an ensemble advanced in one
batch launch per step, the samples read from the device's diagnostics and rotation tracking and the swaths
accumulated on the device (no host copy per step); the checkpoint lines of a series (src/series/checkpoint.ts).
"""
from __future__ import annotations

import base64
import json
import math
import struct
from typing import Callable, Dict, List, Optional, Sequence

import numpy as np

from .runtime import Context, Run
from .scenarios import RunSpec

#: Model seconds between samples (member.ts:28).
SAMPLE_EVERY = 60.0
SWATHS = ("rainTotal", "hailSize", "gustMax", "uhMax")   # checkpoint.ts:11


def _sample(run: Run) -> dict:
    """member.ts:95-99: the domain's strongest values now (no lightning in this configuration: no flashes)."""
    d, r = run.diagnostics(), run.rotation()
    return {"t": run.time, "updraft": d["updraft"], "uh": r["uh"], "rain": d["rainRate"], "gust": d["gust"], "hail": d["hail"],
            "flashes": 0.0, "rotationHeld": r["persisted"], "cores": d["cores"], "outflow": d["outflow"], "outflowLow": d["outflowLow"]}


def run_members(ctx: Context, specs: Sequence[RunSpec], minutes: float, progress: Optional[Callable[[float], None]] = None,
                retire: bool = True) -> List[dict]:
    """runMember (member.ts:93-107) for every spec at once: a sample at the start and every SAMPLE_EVERY model
    seconds, the swaths over the run, the rain gauge and the hail swath at the end; one MemberResult per spec."""
    dts = {s.switches.dt for s in specs}
    if len(dts) != 1:
        raise ValueError("the members of one batch share their step length")
    dt = dts.pop()
    if not all(s.switches.rotation for s in specs):
        raise ValueError("run_members needs the rotation tracking (switches.rotation = 1)")
    runs = [ctx.create(s) for s in specs]
    results = [{"seed": s.seed, "samples": [_sample(r)], "nx": s.grid.nx, "ny": s.grid.ny, "width": s.grid.nx * s.grid.dx,
                "depth": s.grid.ny * s.grid.dy} for s, r in zip(specs, runs)]
    end = minutes * 60
    every = max(1, int(round(SAMPLE_EVERY / dt)))
    time = 0.0
    while time < end - 1e-6:
        n = min(every, int(math.ceil((end - time) / dt - 1e-9)))
        ctx.batch_step(runs, n)
        time = runs[0].time
        for res, r in zip(results, runs):
            if r.time - res["samples"][-1]["t"] >= SAMPLE_EVERY - 1e-6:
                res["samples"].append(_sample(r))
        if progress:
            progress(time)
    for res, r in zip(results, runs):
        cols, sw = r.columns(), r.swaths()
        res.update(rainTotal=cols["precipitation"], hailSize=cols["hailSize"], gustMax=sw["gustMax"], uhMax=sw["uhMax"])
        if retire:
            r.retire()
    return results


# ---- the series checkpoint (src/series/checkpoint.ts)

def series_fingerprint(text: str) -> str:
    """FNV-1a over the text's UTF-16 code units, 32 bits, as 8 hex digits (checkpoint.ts:14-18)."""
    h = 0x811c9dc5
    raw = text.encode("utf-16-le")
    for unit in struct.unpack(f"<{len(raw) // 2}H", raw):
        h ^= unit
        h = (h * 0x01000193) & 0xffffffff
    return f"{h:08x}"


def checkpoint_header(text: str, runs: int, version: str) -> str:
    return json.dumps({"checkpoint": 1, "series": series_fingerprint(text), "runs": runs, "version": version}, separators=(",", ":"))


def _b64(a) -> str:
    return base64.b64encode(np.ascontiguousarray(a, dtype="<f4").tobytes()).decode()


def checkpoint_line(index: int, result: dict) -> str:
    """One finished run as a line: the swaths as float32 in base64, so a resumed series gets them bit for bit
    (checkpoint.ts:26-29)."""
    out = {"index": index}
    for k, v in result.items():
        out[k] = _b64(v) if k in SWATHS else (v.tolist() if isinstance(v, np.ndarray) else v)
    return json.dumps(out, separators=(",", ":"))


def read_checkpoint(file: str, text: str, runs: int) -> dict:
    """readCheckpoint (checkpoint.ts:35-51): {"header", "results": {index: result}} or {"error": ...}; a torn line is
    dropped (that run is run again)."""
    lines = [l for l in file.split("\n") if l.strip()]
    try:
        header = json.loads(lines[0] if lines else "")
    except ValueError:
        return {"error": "not a series checkpoint"}
    if not isinstance(header, dict) or header.get("checkpoint") != 1:
        return {"error": "not a series checkpoint"}
    if header.get("series") != series_fingerprint(text) or header.get("runs") != runs:
        return {"error": "the checkpoint belongs to another series file (or the file has changed since)"}
    results: Dict[int, dict] = {}
    for line in lines[1:]:
        try:
            o = json.loads(line)
        except ValueError:
            continue
        index = o.get("index") if isinstance(o, dict) else None
        if not isinstance(index, int) or isinstance(index, bool) or not 0 <= index < runs:
            continue
        rest = {k: v for k, v in o.items() if k != "index"}
        for k in SWATHS:
            if k in rest:
                rest[k] = np.frombuffer(base64.b64decode(rest[k]), dtype="<f4").copy()
        results[index] = rest
    return {"header": header, "results": results}
