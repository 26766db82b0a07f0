"""Writes tests/golden/takahashi_table.json: the Takahashi charging table (cloud-water rows and the 31 x 30 charge
table, fC) read from the reference's src/core/takahashi.ts, so a CPU test can check the table the device and the
oracle compile in (meteolab_gb300/csrc/sg_takahashi.h) entry for entry. Run where the reference tree is present:

    python tests/golden/make_takahashi_fixture.py [reference root, default /root/reference]
"""
import json
import os
import re
import sys


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    src = open(os.path.join(root, "src/core/takahashi.ts")).read()
    lwc = [float(s) for s in re.search(r"TAKAHASHI_LWC = \[([^\]]*)\]", src).group(1).split(",")]
    body = src[src.index("TAKAHASHI_TABLE"):]
    body = body[body.index("= [") + 3:body.index("]\n\n") + 1]
    table = [[float(s) for s in row.split(",")] for row in re.findall(r"\[([^\[\]]*)\]", body)]
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "takahashi_table.json")
    with open(out, "w") as f:
        json.dump({"source": "src/core/takahashi.ts", "lwc": lwc, "table": table}, f)
    print(out, len(lwc), len(table))


if __name__ == "__main__":
    main()
