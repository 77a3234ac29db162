#!/usr/bin/env python3
"""Fixtures for the exporter's downscale (tools/downscale.h), made by the
reference's own code on the development host: the pyramid levels of seeded
synthetic volumes by the reference's ds_downscale2x (oracle/_ref/libdsref.so)
and the archives the reference writer produces from them with the canonical
vc_encode composition (refcodec.ds_encode). The alphas include the exporter's
default (0.5) and one at which a fused and an unfused multiply-add round apart
for some cells.

Output: tests/golden/ds.json
    python tests/golden/gen_ds.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "volume-compressor_gb300"))
import refcodec as R  # noqa: E402
import vc_gb300 as V  # noqa: E402

CASES = [
    # name, dims, seed, target, method, alpha
    ("cbox_97x131x65_t20", (97, 131, 65), 0x5EED0101, 20.0, 1, 0.5),
    ("cbox_128x96x64_t10_a05943", (128, 96, 64), 0x5EED0102, 10.0, 1, 0.5943000316619873),
    ("box_97x131x65_t20", (97, 131, 65), 0x5EED0101, 20.0, 0, 0.5),
    ("cbox_256_t10", (256, 256, 256), 0x5EED0001, 10.0, 1, 0.5),
    ("cbox_64x64x2_t10_a03", (64, 64, 2), 0x5EED0103, 10.0, 1, 0.3),
]


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


def main():
    out = []
    for name, dims, seed, target, method, alpha in CASES:
        vol = V.synth(*dims, seed)
        data, q0, lods = R.ds_encode(vol, target, method, alpha)
        out.append({"name": name, "dims": list(dims), "seed": seed, "target": target, "method": method,
                    "alpha": alpha, "q0": q0, "len": len(data), "sha256": sha(data),
                    "level_sha256": [sha(l) for l in lods[1:]]})
        print(name, len(data), out[-1]["sha256"][:16])
    with open(os.path.join(HERE, "ds.json"), "w") as f:
        json.dump({"generator": "tests/golden/gen_ds.py", "reference_build": "oracle/Makefile ref (libvcref.so, libdsref.so)",
                   "cases": out}, f, indent=1)


if __name__ == "__main__":
    main()
