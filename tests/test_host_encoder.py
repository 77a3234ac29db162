"""The GPU's range encoder (rangecoder.cuh rc_encode_levels_warp, the
warp-lockstep encoder, run as one lane) built for the host (tests/
host_encoder.cpp) and checked against the oracle's level encoder
(oracle/vc_oracle.c orc_enc_levels / orc_rc_size, which follow
src/vc/vc.c:344-398, 471-544): the level lists of golden archive atoms, which
must also re-encode to the archive's own coder bytes, and random lists (dense
small levels, sparse levels up to 32767 with long escape suffixes, a single
level at the last scan position, empty atoms). The encoding pass must give the
oracle's bytes, the size-only pass their count, and a pass into a buffer of
half the size the same count with only the first half stored. No GPU needed."""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_archive

IDX = np.arange(32768)
SCAN = np.lexsort((IDX, (IDX >> 10) + ((IDX >> 5) & 31) + (IDX & 31)))


def build(tmp_path_factory, flags, name):
    exe = str(tmp_path_factory.mktemp(name) / name)
    src = os.path.join(ROOT, "tests", "host_encoder.cpp")
    inc = os.path.join(ROOT, "volume-compressor_gb300", "csrc")
    r = subprocess.run(["g++", *flags, "-std=c++17", "-w", "-I", inc, src, "-o", exe], capture_output=True, text=True)
    return exe, r


@pytest.fixture(scope="module", params=["plain", "sanitized"])
def harness(tmp_path_factory, request):
    """The plain build, and one with AddressSanitizer and UBSan (no
    out-of-bounds access or undefined behaviour may show up)."""
    if request.param == "plain":
        exe, r = build(tmp_path_factory, ["-O2"], "host_encoder")
        if r.returncode:
            pytest.fail(r.stderr[-2000:])
        return exe
    exe, r = build(tmp_path_factory, ["-O1", "-g", "-fsanitize=address,undefined", "-fno-omit-frame-pointer",
                                      "-fno-sanitize-recover=undefined"], "host_encoder_san")
    if r.returncode:
        pytest.skip("no AddressSanitizer / UBSan with this compiler: " + r.stderr[-200:])
    return exe


def entries(ls):
    """raster levels -> scan-order entries (position | level << 16)"""
    s = ls[SCAN]
    nz = np.nonzero(s)[0].astype(np.uint32)
    return nz | (s[nz].astype(np.uint16).astype(np.uint32) << 16)


def run(harness, oracle, rasters, tmp_path):
    path = str(tmp_path / "lists.bin")
    with open(path, "wb") as f:
        f.write(struct.pack("<I", len(rasters)))
        for lv in rasters:
            lv = np.ascontiguousarray(lv, np.int16)
            buf = np.zeros(200000, np.uint8)
            n = oracle.lib().orc_enc_levels(lv.ctypes.data, buf.ctypes.data, len(buf))
            assert n > 0 and n == oracle.lib().orc_rc_size(lv.ctypes.data)
            e = entries(lv)
            f.write(struct.pack("<II", len(e), n))
            f.write(e.astype("<u4").tobytes())
            f.write(buf[:n].tobytes())
    r = subprocess.run([harness, path], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return {l.split()[0]: int(l.split()[1]) for l in r.stdout.strip().splitlines()}


def test_golden_atom_levels_reencode(harness, oracle, golden, tmp_path):
    rasters = []
    for name in ("synth_64_t10", "synth_prime_97x131x65_t20", "ref_test_basic", "synth_flat_96x64x33_t100",
                 "extreme_sat", "extreme_voxel"):
        data = load_archive(golden[name])
        a = oracle.Archive(data)
        for lod in range(a.nlod):
            _, (nx, ny, nz) = a.lod_dims(lod)
            for az in range((nz + 31) // 32):
                for ay in range((ny + 31) // 32):
                    for ax in range((nx + 31) // 32):
                        c, off, ln = a.payload_range(lod, az, ay, ax)
                        if ln <= 1:
                            continue
                        st = data[off + 1:off + ln]
                        lv = np.zeros(32768, np.int16)
                        buf = np.frombuffer(st + b"\0" * 8, np.uint8)
                        assert oracle.lib().orc_dec_levels(buf.ctypes.data, len(st), lv.ctypes.data) == 0
                        out = np.zeros(200000, np.uint8)
                        n = oracle.lib().orc_enc_levels(lv.ctypes.data, out.ctypes.data, len(out))
                        assert out[:n].tobytes() == st   # the archive's own bytes
                        rasters.append(lv)
        a.close()
    assert len(rasters) > 300
    assert run(harness, oracle, rasters, tmp_path) == {"write": 0, "size": 0, "capped": 0}


def test_random_level_lists(harness, oracle, tmp_path):
    rng = np.random.default_rng(0xE7C)
    rasters = []
    for _ in range(6):   # dense small levels
        rasters.append(rng.integers(-3, 4, 32768).astype(np.int16))
    for _ in range(6):   # sparse, magnitudes up to the quantiser's clamp (long escapes)
        lv = np.zeros(32768, np.int16)
        pos = rng.choice(32768, int(rng.integers(1, 400)), replace=False)
        lv[pos] = (rng.integers(1, 32768, len(pos)) * rng.choice([-1, 1], len(pos))).astype(np.int16)
        rasters.append(lv)
    for m in (1, 11, 12, 13, 14, 27, 28, 1000, 32767):   # one level at the last scan position
        lv = np.zeros(32768, np.int16)
        lv[SCAN[-1]] = -m if m % 2 else m
        rasters.append(lv)
    lv = np.zeros(32768, np.int16)
    lv[SCAN[0]] = 5   # only the first position
    rasters.append(lv)
    rasters.append(np.full(32768, 32767, np.int16))   # every position at the clamp
    rasters.append(np.zeros(32768, np.int16))          # empty: EOB 0
    assert run(harness, oracle, rasters, tmp_path) == {"write": 0, "size": 0, "capped": 0}
