"""The series checkpoint (src/series/checkpoint.ts) on the CPU: the reference's own cases
(src/series/checkpoint.test.ts) on the host mirror in meteolab_gb300/ensemble.py."""
import numpy as np

from meteolab_gb300.ensemble import checkpoint_header, checkpoint_line, read_checkpoint, series_fingerprint

TEXT = '{"scenario":"Летний день","vary":[["shear_0_6km_ms",[0,20]]],"seeds":[1,2]}'


def result(seed):
    # checkpoint.test.ts:5-9
    return {"seed": seed, "nx": 3, "ny": 2, "width": 3600, "depth": 2250,
            "samples": [{"t": 60, "updraft": 12.5, "uh": 40, "rain": 3, "gust": 9, "hail": 0, "flashes": 0, "rotationHeld": 0,
                         "cores": 1, "outflow": 1.25}],
            "rainTotal": np.array([0, 1.1, 2.2, 3.3, 4.4, np.pi], np.float32), "hailSize": np.zeros(6, np.float32),
            "gustMax": np.array([1e-7, 5, 6, 7, 8, 9], np.float32), "uhMax": np.full(6, 250.5, np.float32)}


def test_gives_back_each_kept_run_bit_for_bit_and_skips_a_torn_last_line():
    file = "\n".join([checkpoint_header(TEXT, 4, "v2.10.1"), checkpoint_line(2, result(7)), checkpoint_line(0, result(8)),
                      checkpoint_line(3, result(9))[:40]])
    read = read_checkpoint(file, TEXT, 4)
    assert "error" not in read
    assert read["header"]["version"] == "v2.10.1"
    assert sorted(read["results"]) == [0, 2]
    r = read["results"][2]
    assert r["seed"] == 7 and r["samples"] == result(7)["samples"]
    assert r["rainTotal"].dtype == np.float32
    for k in ("rainTotal", "gustMax", "uhMax"):
        assert np.array_equal(r[k], result(7)[k]), k


def test_refuses_a_checkpoint_of_another_series_or_run_count():
    file = checkpoint_header(TEXT, 4, "v") + "\n"
    assert "error" in read_checkpoint(file, TEXT + " ", 4)
    assert "error" in read_checkpoint(file, TEXT, 5)
    assert "error" in read_checkpoint('{"a":1}', TEXT, 4)
    fp = series_fingerprint(TEXT)
    assert len(fp) == 8 and all(c in "0123456789abcdef" for c in fp)


def test_fingerprint_is_fnv1a_over_utf16_code_units():
    # FNV-1a of the empty text is the offset basis; "a" (0x61) one round of xor and multiply
    assert series_fingerprint("") == "811c9dc5"
    assert series_fingerprint("a") == f"{((0x811c9dc5 ^ 0x61) * 0x01000193) & 0xffffffff:08x}"
    # a character outside ASCII counts as its UTF-16 code unit, not as its UTF-8 bytes
    assert series_fingerprint("Л") == f"{((0x811c9dc5 ^ 0x041B) * 0x01000193) & 0xffffffff:08x}"
