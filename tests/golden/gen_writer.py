#!/usr/bin/env python3
"""Writer-session fixtures made by the reference's own writer (development
host): each session of writer_script.py runs on oracle/_ref/libvcref.so (the
reference built from its source with its release flags) and the result of
every op is recorded, ending with the file's length and SHA-256.

Output: tests/golden/writer.json
    python tests/golden/gen_writer.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "volume-compressor_gb300"))
import refcodec as R  # noqa: E402
import vc_gb300 as V  # noqa: E402
import writer_script as W  # noqa: E402


def canonical():
    g = {c["name"]: c for c in json.load(open(os.path.join(HERE, "golden.json")))["cases"]}["synth_prime_97x131x65_t20"]
    dims, seed = g["dims"], g["seed"]
    ops = [["create", dims, 20.0]]
    qs = R.lod_qs(g["q0"], g["nlod"])
    ops += [["q", l, q] for l, q in enumerate(qs)]
    pyr = W.pyramid(V.synth(*dims, seed), g["nlod"])
    for l, lv in enumerate(pyr):
        nz, ny, nx = lv.shape
        for az in range((nz + 31) // 32):
            for ay in range((ny + 31) // 32):
                for ax in range((nx + 31) // 32):
                    ops.append(["atom", l, az, ay, ax, ["vol", l, az, ay, ax]])
    ops += [["cov", 0, 0, 0, 0], ["cov", 1, 1, 1, 1], ["dec", 0, 1, 2, 1], ["dec", 2, 0, 0, 0],
            ["dec8", 0, 0, 0, 0], ["dec8", 0, 2, 4, 3], ["dec8", 1, 0, 2, 1], ["close"]]
    return {"name": "canonical_97x131x65_t20", "volume": [dims, seed], "ops": ops,
            "expect_sha256": g["sha256"]}


def mixed():
    v = lambda l, az, ay, ax: ["vol", l, az, ay, ax]
    ops = [
        ["create", [1100, 64, 40], 10.0],
        ["q", 0, 2.0],
        ["atom", 0, 0, 0, 3, v(0, 0, 0, 3)],
        ["atom", 0, 1, 1, 34, v(0, 1, 1, 34)],
        ["atom", 1, 0, 0, 5, v(1, 0, 0, 5)],           # no base_q for LOD 1 yet
        ["q", 1, 3.5],
        ["atom", 1, 0, 0, 5, v(1, 0, 0, 5)],
        ["box", 0, [960, 0, 0, 1088, 64, 32], ["vol", 0]],   # across the x region boundary
        ["atom", 0, 0, 0, 3, ["noise", 1, 256]],        # appended again
        ["atom", 0, 0, 1, 4, ["zero"]],
        ["zatom", 0, 1, 0, 3],
        ["atom", 0, 1, 0, 3, v(0, 1, 0, 3)],
        ["zatom", 0, 0, 0, 3],                          # a present atom marked zero
        ["zregion", 2, 0, 0, 0],
        ["cov", 2, 0, 0, 1],
        ["atom", 2, 0, 0, 1, v(2, 0, 0, 1)],            # no base_q for LOD 2
        ["q", 2, 1.0],
        ["atom", 2, 0, 0, 1, v(2, 0, 0, 1)],            # promotes the known-zero region
        ["cov", 2, 0, 0, 1], ["cov", 2, 0, 0, 2],
        ["zregion", 0, 0, 0, 0],                        # has a block: unchanged
        ["zregion", 0, 0, 0, 7],                        # outside the LOD
        ["zatom", 0, 5, 5, 100],                        # outside the LOD
        ["atom", 0, 2, 0, 0, v(0, 1, 0, 0)],            # az out of range
        ["box", 0, [0, 0, 0, 48, 32, 32], ["vol", 0]],  # not whole atoms
        ["box", 0, [32, 32, 32, 96, 64, 64], ["zero"]],
        ["box", 1, [0, 0, 0, 64, 32, 32], ["const", 7]],
        ["box", 0, [1056, 0, 0, 1152, 32, 32], ["vol", 0]],   # runs past the LOD's atoms
        ["q", 0, 0.7],
        ["atom", 0, 1, 1, 10, v(0, 1, 1, 10)],
        ["atom", 0, 0, 0, 31, ["noise", 2, 40]],
        ["dec", 0, 0, 0, 30], ["dec", 0, 1, 1, 10], ["dec", 0, 0, 1, 4], ["dec", 1, 0, 0, 5],
        ["dec", 2, 0, 0, 1], ["dec", 0, 0, 0, 3], ["dec", 0, 0, 0, 34], ["dec", 0, 2, 0, 0],
        ["dec8", 0, 0, 0, 30], ["dec8", 0, 1, 0, 33], ["dec8", 1, 0, 0, 16], ["dec8", 2, 0, 0, 0],
        ["dec8", 0, 0, 0, 35], ["dec8", 5, 0, 0, 0],
        ["cov", 0, 0, 0, 3], ["cov", 0, 1, 0, 3], ["cov", 0, 0, 1, 4], ["cov", 0, 1, 1, 33],
        ["cov", 0, 0, 0, 35], ["cov", 0, 5, 5, 100], ["cov", 1, 0, 0, 1], ["cov", 0, 1, 1, 2],
        ["close"],
    ]
    return {"name": "mixed_1100x64x40", "volume": [[1100, 64, 40], 0x5EED0201], "ops": ops}


def zero():
    ops = [
        ["create", [64, 64, 64], 30.0],
        ["atom", 0, 0, 0, 0, ["zero"]],
        ["atom", 0, 0, 0, 1, ["vol", 0, 0, 0, 1]],
        ["box", 0, [0, 0, 0, 64, 64, 64], ["zero"]],
        ["zregion", 1, 0, 0, 0],
        ["cov", 0, 1, 1, 1], ["cov", 1, 0, 0, 0],
        ["dec", 0, 0, 0, 0], ["dec8", 0, 0, 0, 0],
        ["q", 0, 1.0],
        ["box", 0, [0, 0, 0, 64, 64, 64], ["vol", 0]],
        ["dec8", 0, 0, 0, 0], ["dec8", 0, 1, 1, 1],
        ["q", 1, 0.01], ["atom", 1, 0, 0, 0, ["vol", 1, 0, 0, 0]],   # q clamped to 0.05
        ["dec", 1, 0, 0, 0],
        ["close"],
    ]
    return {"name": "zero_64", "volume": [[64, 64, 64], 0x5EED0202], "ops": ops}


def marks():
    ops = [
        ["create", [300, 2100, 90], 12.0],
        ["zatom", 0, 0, 0, 0], ["zatom", 0, 2, 40, 9], ["zregion", 0, 0, 1, 0], ["zatom", 0, 1, 33, 1],
        ["zregion", 1, 0, 0, 0], ["zregion", 1, 0, 0, 0], ["zatom", 3, 0, 1, 0], ["q", 2, 5.0], ["q", 9, 1.0],
        ["zregion", 0, 3, 3, 3],
        ["cov", 0, 0, 0, 0], ["cov", 0, 2, 40, 9], ["cov", 0, 1, 33, 1], ["cov", 0, 1, 40, 1], ["cov", 1, 0, 5, 0],
        ["cov", 0, 0, 0, 1], ["cov", 3, 0, 1, 0], ["cov", 7, 0, 0, 0],
        ["close"],
    ]
    return {"name": "marks_300x2100x90", "volume": [[8, 8, 8], 1], "ops": ops}


def main():
    L = W.bind(R.lib())
    sessions = [canonical(), mixed(), zero(), marks()]
    for s in sessions:
        s["results"] = W.run(L, s, V.synth)
        if "expect_sha256" in s:
            assert s["results"][-1][1] == s["expect_sha256"], s["name"]
        print(s["name"], len(s["ops"]), "ops", s["results"][-1])
    with open(os.path.join(HERE, "writer.json"), "w") as f:
        json.dump({"generator": "tests/golden/gen_writer.py", "reference_build": "oracle/Makefile ref (libvcref.so)",
                   "sessions": sessions}, f)


if __name__ == "__main__":
    main()
