"""The GPU's range decoders (rangecoder.cuh: latency, staged latency, compact
scalar, warp-lockstep and per-lane) built for the host with single-lane
stand-ins for the CUDA intrinsics (tests/host_decoders.cpp) and checked
against the oracle's level decoder (oracle/vc_oracle.c::orc_dec_levels, which
follows src/vc/vc.c:545-560) on every atom stream of the golden archives, on
streams of coded noise with escapes, on truncated streams, on random byte
streams and on crafted streams with over-long escape prefixes. No GPU needed."""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, load_archive
from rcstream import hostile_payload

IDX = np.arange(32768)
SCAN = np.lexsort((IDX, (IDX >> 10) + ((IDX >> 5) & 31) + (IDX & 31)))   # frequency, then raster


def expected(oracle, stream):
    lv = np.zeros(32768, np.int16)
    buf = np.frombuffer(bytes(stream) + b"\0" * 8, np.uint8)
    bad = oracle.lib().orc_dec_levels(buf.ctypes.data, len(stream), lv.ctypes.data)
    ls = lv[SCAN]
    nz = np.nonzero(ls)[0].astype(np.uint32)
    ent = nz | (ls[nz].astype(np.uint16).astype(np.uint32) << 16)
    return int(bad != 0), ent


def atom_streams(oracle, data):
    a = oracle.Archive(data)
    out = []
    for lod in range(a.nlod):
        _, (nx, ny, nz) = a.lod_dims(lod)
        for az in range((nz + 31) // 32):
            for ay in range((ny + 31) // 32):
                for ax in range((nx + 31) // 32):
                    cov, off, ln = a.payload_range(lod, az, ay, ax)
                    if ln > 1:
                        out.append(bytes(data[off + 1:off + ln]))
    a.close()
    return out


SANITIZE = ["-O1", "-g", "-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-fno-sanitize-recover=undefined"]


def build(tmp_path_factory, flags, name):
    exe = str(tmp_path_factory.mktemp(name) / name)
    src = os.path.join(ROOT, "tests", "host_decoders.cpp")
    inc = os.path.join(ROOT, "volume-compressor_gb300", "csrc")
    r = subprocess.run(["g++", *flags, "-std=c++17", "-w", "-I", inc, src, "-o", exe], capture_output=True, text=True)
    return exe, r


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe, r = build(tmp_path_factory, ["-O2"], "host_decoders")
    if r.returncode:
        pytest.fail(r.stderr[-2000:])
    return exe


def run(harness, oracle, streams, tmp_path):
    path = str(tmp_path / "streams.bin")
    with open(path, "wb") as f:
        f.write(struct.pack("<I", len(streams)))
        for s in streams:
            bad, ent = expected(oracle, s)
            f.write(struct.pack("<III", len(s), bad, len(ent)))
            f.write(s)
            f.write(ent.astype("<u4").tobytes())
    r = subprocess.run([harness, path], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    rows = [line.split() for line in r.stdout.strip().splitlines()]
    return {name: int(diff) for name, diff, _ in rows}


def golden_streams(oracle, golden):
    streams = []
    for name in ("synth_64_t10", "synth_prime_97x131x65_t20", "synth_flat_96x64x33_t100", "ref_test_basic",
                 "extreme_sat", "extreme_line", "extreme_voxel", "tiny_1x1x1"):
        streams += atom_streams(oracle, load_archive(golden[name]))
    return streams


def test_golden_archive_streams(harness, oracle, golden, tmp_path):
    streams = golden_streams(oracle, golden)
    assert len(streams) > 300
    assert run(harness, oracle, streams, tmp_path) == dict.fromkeys(
        ("latency", "staged", "scalar", "lockstep", "per-lane"), 0)


def other_streams(oracle):
    rng = np.random.default_rng(0xDEC0DE)
    vol = rng.integers(0, 256, (64, 64, 64)).astype(np.uint8)
    s, data = oracle.encode_fixed_q(vol, 1.0, [0.05] * 8)   # the largest levels: many escapes
    assert s == 0
    coded = atom_streams(oracle, data)
    streams = list(coded)
    for c in coded[:6]:   # cut short: the bytes past the end read as zero
        for n in (1, 5, 6, len(c) // 3, len(c) // 2, len(c) - 1):
            streams.append(c[:n])
    for n in list(range(0, 24)) + [64, 300, 1000, 4000]:   # random bytes
        for _ in range(3):
            streams.append(rng.integers(0, 256, n).astype(np.uint8).tobytes())
    for ones in (31, 32, 33, 40):   # escape prefixes at and past the limit
        streams.append(hostile_payload(prefix_ones=ones)[1:])
    return streams


def test_noise_escapes_truncation_and_random_streams(harness, oracle, tmp_path):
    streams = other_streams(oracle)
    bad = [expected(oracle, s)[0] for s in streams]
    assert sum(bad) >= 2 and sum(bad) < len(streams)
    assert run(harness, oracle, streams, tmp_path) == dict.fromkeys(
        ("latency", "staged", "scalar", "lockstep", "per-lane"), 0)


def test_all_streams_under_sanitizers(oracle, golden, tmp_path_factory, tmp_path):
    """Both stream sets through a build with AddressSanitizer and UBSan: no
    out-of-bounds access and no undefined behaviour in any decoder (this found
    the per-lane decoder reading one entry past the band table)."""
    exe, r = build(tmp_path_factory, SANITIZE, "host_decoders_san")
    if r.returncode:
        pytest.skip("no AddressSanitizer / UBSan with this compiler: " + r.stderr[-200:])
    assert run(exe, oracle, golden_streams(oracle, golden) + other_streams(oracle), tmp_path) == dict.fromkeys(
        ("latency", "staged", "scalar", "lockstep", "per-lane"), 0)
