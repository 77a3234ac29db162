#!/usr/bin/env python3
"""v2 container fixtures made by the reference itself.

Each stored v1 golden archive is rewritten into the v2 container by the
reference's repack tool (tools/vc_repack.c, built from its sources by
`make -C oracle repack` into oracle/_ref/vc_repack). The v2 bytes are stored
xz-compressed as tests/golden/v2_<case>.vca.xz and listed with their SHA-256 in
tests/golden/v2.json. Run from the repository root where the reference checkout
exists; the fixtures then travel with the repository.
"""
import hashlib
import json
import lzma
import os
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
GOLDEN = os.path.join(ROOT, "tests", "golden")
TOOL = os.path.join(ROOT, "oracle", "_ref", "vc_repack")


def main():
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "repack"], check=True, capture_output=True)
    cases = json.load(open(os.path.join(GOLDEN, "golden.json")))["cases"]
    out = []
    with tempfile.TemporaryDirectory() as td:
        for c in cases:
            if not c.get("file"):
                continue
            v1 = lzma.decompress(open(os.path.join(GOLDEN, c["file"]), "rb").read())
            src, dst = os.path.join(td, "in.vca"), os.path.join(td, "out.vca")
            open(src, "wb").write(v1)
            r = subprocess.run([TOOL, src, dst, "--threads", "4"], capture_output=True, text=True)
            if r.returncode != 0:
                sys.exit(f"repack failed for {c['name']}: {r.stderr}")
            v2 = open(dst, "rb").read()
            name = f"v2_{c['name']}.vca.xz"
            open(os.path.join(GOLDEN, name), "wb").write(lzma.compress(v2, preset=9))
            out.append({"name": c["name"], "v1_file": c["file"], "file": name, "len": len(v2),
                        "sha256": hashlib.sha256(v2).hexdigest()})
            print(c["name"], len(v1), "->", len(v2))
    json.dump({"generator": "tests/golden/gen_v2.py (reference tools/vc_repack.c)", "cases": out},
              open(os.path.join(GOLDEN, "v2.json"), "w"), indent=1)


if __name__ == "__main__":
    main()
