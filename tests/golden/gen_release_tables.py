#!/usr/bin/env python3
"""Pin the float tables of the reference's release build (x86-64 host only).

The reference computes its quantizer steps with ``powf`` inside a loop that
gcc vectorises under its release flags (src/vc/vc.c:273-279, CMakeLists.txt:46),
and divides by the step with an RCPPS estimate plus one Newton step
(src/vc/vc.c:299). Neither is reproducible from the source text alone, so this
script measures both on the host that produces the golden archives and writes
them as data into ``volume-compressor_gb300/csrc/vc_release_tables.h``:

* ``vc_step_base_bits[f]`` / ``vc_step_alt_bits[f]``: the (at most two) float
  values the release build stores in ``g_step`` for L1 frequency f, and
  ``vc_step_alt_mask``: one bit per raster index selecting the alternate value.
* ``vc_rcp_est_bits[t]``: RCPPS(1 + t/2048), t = 0..2047.

Requires oracle/_ref/libvcref.so (``make -C oracle ref``) and an x86-64 CPU.
"""
import ctypes
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(ROOT, "volume-compressor_gb300", "csrc", "vc_release_tables.h")


def step_tables():
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libvcref.so"))
    st = np.zeros(32768, np.float32)
    cm = np.zeros(1024, np.int32)
    lib.refshim_tables(cm.ctypes.data_as(ctypes.c_void_p), st.ctypes.data_as(ctypes.c_void_p), None)
    bits = st.view(np.uint32)
    idx = np.arange(32768)
    freq = idx // 1024 + (idx // 32) % 32 + idx % 32
    base = np.zeros(94, np.uint32)
    alt = np.zeros(94, np.uint32)
    mask = np.zeros(32768, bool)
    for f in range(94):
        sel = np.nonzero(freq == f)[0]
        vals = bits[sel]
        base[f] = vals[0]
        others = np.unique(vals[vals != base[f]])
        if len(others) > 1:
            sys.exit(f"frequency {f}: more than two step values {others}")
        alt[f] = others[0] if len(others) else base[f]
        mask[sel] = vals != base[f]
    words = np.packbits(mask.reshape(-1, 8)[:, ::-1], axis=1).reshape(-1)  # LSB-first bytes
    words = words.view(np.uint32)  # little-endian: bit i of word w = raster index 32*w+i
    return base, alt, words, cm.reshape(32, 32)


def rcp_table():
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "rcp_probe")
        subprocess.check_call(["gcc", "-O2", "-o", exe, os.path.join(HERE, "rcp_probe.c")])
        out = subprocess.check_output([exe]).decode().split()
    tab = np.array([int(v) for v in out], np.uint32)
    assert len(tab) == 2048
    return tab


def fmt(name, arr, per_line=8):
    lines = []
    for i in range(0, len(arr), per_line):
        lines.append("    " + ", ".join(f"0x{int(v):08x}u" for v in arr[i:i + per_line]) + ",")
    return f"static const uint32_t {name}[{len(arr)}] = {{\n" + "\n".join(lines) + "\n};\n"


def main():
    base, alt, mask, cm = step_tables()
    rcp = rcp_table()
    hdr = [
        "// Generated by tests/golden/gen_release_tables.py from the reference's release",
        "// build (gcc -O3 -ffast-math -march=native, x86-64). Do not edit by hand.",
        "//",
        "// g_step (src/vc/vc.c:273-279) is powf(1+f, 0.65f) for L1 frequency f of a raster",
        "// index; the release build's vectorised loop stores one of at most two",
        "// neighbouring floats per frequency, chosen by raster position. The quantizer",
        "// (src/vc/vc.c:299) divides by the step with the RCPPS estimate refined by one",
        "// Newton step; vc_rcp_est_bits[t] = RCPPS(1 + t/2048) as measured on the host",
        "// that produced the golden archives (a function of the top 11 mantissa bits",
        "// that scales exactly with the exponent).",
        "#ifndef VC_RELEASE_TABLES_H",
        "#define VC_RELEASE_TABLES_H",
        "#include <stdint.h>",
        "#define VC_NFREQ 94",
        fmt("vc_step_base_bits", base),
        fmt("vc_step_alt_bits", alt),
        "// bit (i & 31) of word (i >> 5) set: raster index i uses vc_step_alt_bits[freq(i)]",
        fmt("vc_step_alt_mask", mask),
        fmt("vc_rcp_est_bits", rcp),
        "// CMATA (src/vc/vc.c:75-88): round(c_k cos(pi (2n+1) k / 64) 2^14), row k = frequency",
        "#define VC_CMAT_INIT { \\",
        "\n".join("    {" + ", ".join(str(int(v)) for v in row) + "}, \\" for row in cm),
        "}",
        "#endif",
        "",
    ]
    with open(OUT, "w") as f:
        f.write("\n".join(hdr))
    print("wrote", OUT, "alt positions:", int(np.unpackbits(mask.view(np.uint8)).sum()))


if __name__ == "__main__":
    main()
