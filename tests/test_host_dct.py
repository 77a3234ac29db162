"""The device's exact DCT-32 line transforms (dct32.cuh: the recursive even/odd
butterfly, 342-344 multiplies per line instead of 1024) built for the host
(tests/host_dct.cpp) and run in the transform kernels' pass order (x, y, z)
over whole atoms, against the oracle's atom transforms (oracle/vc_oracle.c
orc_fdct / orc_idct, which follow src/vc/vc.c:142-229): forward coefficients
of synthetic and random atoms at their own dc and at extreme centres; inverse
voxels of real coefficient fields (dequantised levels of golden archives),
of random fields that leave most voxels unclamped, and of hostile fields whose
sums wrap around i32. No GPU needed."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_archive

IDX = np.arange(32768)
SCAN = np.lexsort((IDX, (IDX >> 10) + ((IDX >> 5) & 31) + (IDX & 31)))


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("host_dct") / "host_dct")
    src = os.path.join(ROOT, "tests", "host_dct.cpp")
    inc = os.path.join(ROOT, "volume-compressor_gb300", "csrc")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-w", "-I", inc, src, "-o", exe], capture_output=True, text=True)
    if r.returncode:
        pytest.fail(r.stderr[-2000:])
    return exe


def run(harness, mode, recs, tmp_path):
    fi, fo = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    with open(fi, "wb") as f:
        for dc, arr in recs:
            f.write(np.int32(dc).tobytes())
            f.write(np.ascontiguousarray(arr).tobytes())
    r = subprocess.run([harness, mode, fi, fo], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    dt = np.uint8 if mode == "inv" else np.int32
    return np.fromfile(fo, dt).reshape(len(recs), 32768)


def test_forward_matches_oracle(vc, oracle, harness, tmp_path):
    rng = np.random.default_rng(0xF0D)
    vol = vc.synth(64, 64, 32, vc.config_seed(3))
    atoms = [np.ascontiguousarray(vol[:, y:y + 32, x:x + 32]).ravel() for y in (0, 32) for x in (0, 32)]
    atoms += [rng.integers(0, 256, 32768).astype(np.uint8) for _ in range(4)]
    atoms += [np.full(32768, 255, np.uint8), np.zeros(32768, np.uint8),
              (np.indices((32, 32, 32)).sum(0) % 2 * 255).astype(np.uint8).ravel()]   # checkerboard
    recs = []
    for a in atoms:
        dc = (int(a.astype(np.int64).sum()) + 16384) // 32768   # src/vc/vc.c:603
        recs += [(dc, a), (0, a), (255, a)]
    got = run(harness, "fwd", recs, tmp_path)
    for i, (dc, a) in enumerate(recs):
        want = np.zeros(32768, np.int32)
        oracle.lib().orc_fdct(a.ctypes.data, dc, want.ctypes.data)
        assert np.array_equal(got[i], want), i


def test_inverse_matches_oracle(oracle, golden, harness, tmp_path):
    rng = np.random.default_rng(0x1DC7)
    recs = []
    # real fields: the dequantised levels of golden archive atoms
    data = load_archive(golden["synth_prime_97x131x65_t20"])
    a = oracle.Archive(data)
    q = a.base_q(0)
    lv = np.zeros(32768, np.int16)
    for az, ay, ax in ((0, 0, 0), (1, 2, 1), (0, 3, 2), (1, 4, 3)):
        c, off, ln = a.payload_range(0, az, ay, ax)
        if ln <= 1:
            continue
        st = np.frombuffer(data[off + 1:off + ln] + b"\0" * 8, np.uint8)
        assert oracle.lib().orc_dec_levels(st.ctypes.data, ln - 1, lv.ctypes.data) == 0
        coef = np.zeros(32768, np.int32)
        oracle.lib().orc_dequantize(lv.ctypes.data, np.float32(q), coef.ctypes.data)
        recs.append((data[off], coef))
    a.close()
    assert len(recs) >= 3
    # random fields, small enough that most voxels stay inside [0, 255]
    for s in (40, 400, 4000):
        recs.append((128, rng.integers(-s, s + 1, 32768).astype(np.int32)))
    # energy only at low frequencies (a smooth atom)
    low = np.zeros(32768, np.int32)
    lowi = IDX[((IDX >> 10) < 4) & (((IDX >> 5) & 31) < 4) & ((IDX & 31) < 4)]
    low[lowi] = rng.integers(-3000, 3001, len(lowi))
    recs.append((100, low))
    # hostile fields: sums that wrap around i32 in every pass
    for s in (1 << 20, 1 << 26, (1 << 31) - 1):
        recs.append((0, rng.integers(-s, s, 32768, dtype=np.int64).astype(np.int32)))
    recs.append((7, np.full(32768, np.iinfo(np.int32).min, np.int32)))
    recs.append((250, np.full(32768, np.iinfo(np.int32).max, np.int32)))
    got = run(harness, "inv", recs, tmp_path)
    unclamped = 0
    for i, (dc, coef) in enumerate(recs):
        want = np.zeros(32768, np.uint8)
        oracle.lib().orc_idct(np.ascontiguousarray(coef).ctypes.data, int(dc), want.ctypes.data)
        assert np.array_equal(got[i], want), i
        unclamped += int(((want > 0) & (want < 255)).sum())
    assert unclamped > 32768 * 3   # the comparison sees real values, not only the clamp
