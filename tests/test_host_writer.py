"""The writer (volume-compressor_gb300/csrc/vc_writer.c) and the host reader
(vc_host.c) built for the host with a stand-in device layer (tests/
host_writer.c): atom batches are encoded by the oracle's atom encoder, whose
payloads are the reference's, so every other byte of the file (region index,
slot blocks, payload placement, zero marks, base_q table, close) is this
library's own host code. Writer sessions without read-backs then run on it
and, live, on the reference's own writer (oracle/_ref, this host only):
the stored sessions of tests/golden/writer.json and random sessions of atom
and box appends (aligned and not, in and past every LOD, zero, constant, noise
and volume contents), zero marks, base_q settings and coverage queries, with
the appends made one at a time (every op's result and the closed file's bytes
must be the reference's) and through the asynchronous queue, which reports a
failed append at the next flush instead (the closed file must be the
reference's). No GPU needed."""
import ctypes
import json
import os
import subprocess

import numpy as np
import pytest

import writer_script as W
from conftest import GOLDEN, ROOT


@pytest.fixture(scope="module")
def host_writer(tmp_path_factory, oracle):
    so = str(tmp_path_factory.mktemp("host_writer") / "libhostwriter.so")
    csrc = os.path.join(ROOT, "volume-compressor_gb300", "csrc")
    odir = os.path.join(ROOT, "oracle")
    r = subprocess.run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-I", os.path.join(ROOT, "include"),
                        "-I", csrc, "-I", odir, os.path.join(ROOT, "tests", "host_writer.c"),
                        os.path.join(csrc, "vc_writer.c"), os.path.join(csrc, "vc_host.c"), "-o", so,
                        "-L", odir, "-loracle", "-Wl,-rpath," + odir, "-Wl,--no-undefined", "-lpthread", "-lm"],
                       capture_output=True, text=True)
    if r.returncode:
        pytest.fail(r.stderr[-2000:])
    return W.bind(ctypes.CDLL(so))


@pytest.fixture(scope="module")
def ref_writer():
    import refcodec
    if not refcodec.available():
        pytest.skip("reference build (oracle/_ref) not present on this host")
    return W.bind(ctypes.CDLL(refcodec.REF_SO))   # own handle: the script's ctypes types


def without_readback(session):
    return {"volume": session["volume"], "ops": [o for o in session["ops"] if o[0] not in ("dec", "dec8")]}


def test_stored_sessions(vc, host_writer, ref_writer):
    for s in json.load(open(os.path.join(GOLDEN, "writer.json")))["sessions"]:
        ss = without_readback(s)
        want = W.run(ref_writer, ss, vc.synth)
        assert W.run(host_writer, ss, vc.synth) == want, s["name"]
        # queued appends report a failure at the next flush instead: the file is the same
        assert W.run(host_writer, ss, vc.synth, async_atoms=True)[-1] == want[-1], s["name"]


def random_session(rng):
    dims = [int(rng.integers(1, 300)) for _ in range(3)]
    ops = [["create", dims, float(rng.choice([5.0, 12.0, 40.0]))]]
    nlod = 1
    while max((d + (1 << nlod) - 1) >> nlod for d in dims) > 1 and nlod < 8:
        nlod += 1
    for _ in range(int(rng.integers(5, 40))):
        lod = int(rng.choice([0, 0, 0, 1, 2, nlod - 1, nlod, -1]))
        l = max(0, min(lod, nlod - 1))
        d = [max(1, (v + (1 << l) - 1) >> l) for v in dims]
        past = int(rng.integers(0, 4) == 0)   # x, y, z atom; a quarter of them may lie one past the edge
        at = [int(rng.integers(0, (v + 31) // 32 + past)) for v in d]
        src = [["vol", l, at[2], at[1], at[0]], ["zero"], ["const", int(rng.integers(1, 256))],
               ["noise", int(rng.integers(0, 1 << 30)), int(rng.choice([2, 16, 256]))]][int(rng.integers(0, 4))]
        k = int(rng.integers(0, 12))
        if k < 4:
            ops.append(["atom", lod, at[2], at[1], at[0], src])
        elif k < 6:
            b0 = []
            for v in d:   # mostly atom-aligned starts
                x = int(rng.integers(0, v))
                b0.append(x - x % 32 if rng.integers(0, 4) else x)
            if rng.integers(0, 2):   # whole atoms, inside the LOD
                b0 = [b - b % 32 for b in b0]
                b1 = [min(v, b + 32 * int(rng.integers(1, 4))) for v, b in zip(d, b0)]
            else:
                b1 = [min(v + int(rng.integers(0, 2)) * 7, b + int(rng.integers(1, 80))) for v, b in zip(d, b0)]
            box = [b0[0], b0[1], b0[2], b1[0], b1[1], b1[2]]
            bsrc = ["vol", l] if src[0] == "vol" else src
            ops.append(["box", lod, box, bsrc])
        elif k < 7:
            ops.append(["zatom", lod, at[2], at[1], at[0]])
        elif k < 8:
            ops.append(["zregion", lod, 0, int(rng.integers(0, 2)), 0])
        elif k < 9:
            ops.append(["q", lod, float(rng.choice([0.01, 0.5, 2.0, 9.0, 5000.0]))])
        else:
            ops.append(["cov", lod, at[2], at[1], at[0]])
    ops.append(["close"])
    return {"volume": [dims, int(rng.integers(1, 1 << 30))], "ops": ops}


def test_random_sessions(vc, host_writer, ref_writer):
    rng = np.random.default_rng(0x4B17E)
    appended = 0
    for trial in range(24):
        s = random_session(rng)
        want = W.run(ref_writer, s, vc.synth)
        assert W.run(host_writer, s, vc.synth) == want, (trial, s)
        assert W.run(host_writer, s, vc.synth, async_atoms=True)[-1] == want[-1], (trial, s)
        appended += sum(1 for o, r in zip(s["ops"], want) if o[0] in ("atom", "box") and r == 0)
    assert appended > 30


def build_mt(tmp, oracle, sanitize=None):
    exe = str(tmp / ("host_writer_mt_" + (sanitize or "plain").replace(",", "_")))
    csrc = os.path.join(ROOT, "volume-compressor_gb300", "csrc")
    odir = os.path.join(ROOT, "oracle")
    flags = ["-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=" + sanitize] if sanitize else ["-O2"]
    r = subprocess.run(["gcc", *flags, "-std=gnu11", "-I", os.path.join(ROOT, "include"), "-I", csrc, "-I", odir,
                        os.path.join(ROOT, "tests", "host_writer_mt.c"), os.path.join(ROOT, "tests", "host_writer.c"),
                        os.path.join(csrc, "vc_writer.c"), os.path.join(csrc, "vc_host.c"), "-L", odir, "-loracle",
                        "-Wl,-rpath," + odir, "-lpthread", "-lm", "-o", exe], capture_output=True, text=True)
    return exe, r


def test_concurrent_appends(oracle, tmp_path):
    """Threads (1, 4 and 16) append every atom of two LODs of a volume spanning
    three regions, in shuffled orders, synchronously, queued and as zero marks,
    with coverage queries between: every atom of the closed file has the
    coverage it was given and decodes (oracle's reader) to what the oracle's
    own encode and decode of its source give (tests/host_writer_mt.c)."""
    exe, r = build_mt(tmp_path, oracle)
    assert r.returncode == 0, r.stderr[-2000:]
    for threads in (1, 4, 16):
        r = subprocess.run([exe, str(tmp_path / f"mt{threads}.vca"), str(threads)], capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0 and r.stdout.strip() == "atoms 462 wrong 0" and not r.stderr, (threads, r.stdout,
                                                                                                 r.stderr[-2000:])


def test_concurrent_appends_race_free(oracle, tmp_path):
    """The same with 8 threads under ThreadSanitizer: no data race in the
    writer's batching, index, slot and cursor updates."""
    exe, r = build_mt(tmp_path, oracle, "thread")
    if r.returncode:
        pytest.skip("no ThreadSanitizer with this compiler: " + r.stderr[-200:])
    r = subprocess.run([exe, str(tmp_path / "mt.vca"), "8"], capture_output=True, text=True, timeout=900)
    if "FATAL: ThreadSanitizer" in r.stderr:
        pytest.skip(r.stderr.strip().splitlines()[0])
    assert "WARNING: ThreadSanitizer" not in r.stderr, r.stderr[:4000]
    assert r.returncode == 0 and r.stdout.strip() == "atoms 462 wrong 0", r.stdout + r.stderr[-2000:]


def test_concurrent_appends_memory_clean(oracle, tmp_path):
    """The same with 8 threads under AddressSanitizer and UBSan: no invalid
    access, no undefined behaviour and nothing leaked at exit."""
    exe, r = build_mt(tmp_path, oracle, "address,undefined")
    if r.returncode:
        pytest.skip("no AddressSanitizer with this compiler: " + r.stderr[-200:])
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="print_stacktrace=1")
    r = subprocess.run([exe, str(tmp_path / "mt.vca"), "8"], capture_output=True, text=True, timeout=900, env=env)
    assert "runtime error" not in r.stderr and "ERROR: " not in r.stderr, r.stderr[:4000]
    assert r.returncode == 0 and r.stdout.strip() == "atoms 462 wrong 0", r.stdout + r.stderr[-2000:]
