"""The writer API (vc_create, vc_set_base_q, vc_append_atom, vc_append_box,
vc_mark_zero_atom / _region, vc_writer_decode_atom / _coverage /
_decode_2x2x2, vc_writer_close; src/vc/vc.c:995-1245, 1475-1530) with the
encoding on the GPU.

Sessions of writer calls (tests/golden/writer_script.py) were run on the
reference's own writer (tests/golden/gen_writer.py). Replayed here, every op
must give the reference's result: its status, its reads (coverage and
decoded bytes), and the file's bytes at close. The canonical session also
reproduces the stored archive of that volume. The marks-only session needs
no GPU. Concurrent appends from several threads lay out in a different
order, but must decode to the same volume."""
import ctypes
import hashlib
import json
import os
import threading

import numpy as np
import pytest

import writer_script as W
from conftest import GOLDEN, load_archive

SESS = {s["name"]: s for s in json.load(open(os.path.join(GOLDEN, "writer.json")))["sessions"]}


def mylib(vc):
    return W.bind(ctypes.CDLL(vc.LIB_PATH))   # own handle: the script's ctypes types


def test_marks_session_matches_reference(vc):
    s = SESS["marks_300x2100x90"]
    assert W.run(mylib(vc), s, vc.synth) == s["results"]


def test_writer_argument_checks(vc, tmp_path):
    L = mylib(vc)
    p = str(tmp_path / "a.vca").encode()
    assert not L.vc_create(p, W.Dims(0, 4, 4), 10.0)
    assert not L.vc_create(p, W.Dims(4, 4, 4), 0.5)
    assert not L.vc_create(str(tmp_path / "missing" / "a.vca").encode(), W.Dims(4, 4, 4), 10.0)
    w = L.vc_create(p, W.Dims(40, 40, 40), 10.0)
    assert w
    assert L.vc_set_base_q(w, 6, 1.0) == 0 and L.vc_set_base_q(w, 7, 1.0) == 2   # 40 -> 1: 7 LODs
    assert L.vc_set_base_q(w, 0, float("nan")) == 2
    a = np.zeros(32768, np.uint8)
    assert L.vc_append_atom(w, 0, 0, 0, 2, a.ctypes.data) == 2
    assert L.vc_append_atom(w, 7, 0, 0, 0, a.ctypes.data) == 2
    assert L.vc_append_box(w, 0, W.Box(0, 0, 0, 32, 32, 16), a.ctypes.data) == 2
    assert L.vc_append_box(w, 0, W.Box(32, 0, 0, 32, 32, 32), a.ctypes.data) == 2
    assert L.vc_writer_coverage(w, 0, 0, 0, 0) == 0
    L.vc_writer_close(w)
    L.vc_writer_close(None)
    data = open(p, "rb").read()
    assert len(data) == 128 + 1024 * 16 and data[:4] == b"VC1\x00"


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["canonical_97x131x65_t20", "mixed_1100x64x40", "zero_64"])
def test_gpu_session_matches_reference(vc, gpu, name):
    s = SESS[name]
    got = W.run(mylib(vc), s, vc.synth)
    for i, (op, g, want) in enumerate(zip(s["ops"], got, s["results"])):
        assert g == want, (i, op)
    if "expect_sha256" in s:
        assert got[-1][1] == s["expect_sha256"]


@pytest.mark.gpu
def test_gpu_async_session_matches_reference(vc, gpu):
    """The canonical session with every atom queued asynchronously (one large
    batch, flushed before the reads): the reference's bytes and reads."""
    s = SESS["canonical_97x131x65_t20"]
    got = W.run(mylib(vc), s, vc.synth, async_atoms=True)
    assert got == s["results"]


@pytest.mark.gpu
def test_gpu_async_errors_counted_at_flush(vc, gpu, tmp_path):
    with vc.Writer(str(tmp_path / "e.vca"), (64, 64, 64), 10.0) as w:
        noise = np.random.default_rng(1).integers(0, 255, 32768, dtype=np.uint8)
        assert w.append_atom_async(0, 0, 0, 0, noise) == 0          # no base_q yet: fails at flush
        assert w.append_atom_async(0, 0, 0, 1, np.zeros(32768, np.uint8)) == 0
        assert w.append_atom_async(0, 0, 0, 2, noise) == vc.VC_ERR_RANGE   # outside: at once
        assert w.flush() == (vc.VC_ERR_RANGE, 1)
        assert w.flush() == (0, 0)
        assert w.coverage(0, 0, 0, 0) == 0 and w.coverage(0, 0, 0, 1) == 1
        assert w.set_base_q(0, 2.0) == 0
        for i in range(9000):   # crosses the automatic commit
            assert w.append_atom_async(0, i % 2, (i // 2) % 2, 1, noise) == 0
        assert w.flush() == (0, 0)
        assert w.coverage(0, 1, 0, 1) == 2


@pytest.mark.gpu
@pytest.mark.parametrize("threads", [4, 16])
def test_gpu_concurrent_appends_decode_like_canonical(vc, gpu, golden, tmp_path, threads):
    """Atoms of every LOD appended from several threads at once (batched
    together on the device): the layout differs from the single-threaded
    reference, the decoded volume must not."""
    g = golden["synth_prime_97x131x65_t20"]
    import refcodec
    pyr = W.pyramid(vc.synth(*g["dims"], g["seed"]), g["nlod"])
    qs = refcodec.lod_qs(g["q0"], g["nlod"])
    jobs = []
    for l, lv in enumerate(pyr):
        nz, ny, nx = lv.shape
        for az in range((nz + 31) // 32):
            for ay in range((ny + 31) // 32):
                for ax in range((nx + 31) // 32):
                    jobs.append((l, az, ay, ax, np.ascontiguousarray(W.region_of(
                        lv, ax * 32, ay * 32, az * 32, ax * 32 + 32, ay * 32 + 32, az * 32 + 32))))
    np.random.default_rng(threads).shuffle(jobs)
    path = str(tmp_path / "c.vca")
    with vc.Writer(path, g["dims"], 20.0) as w:
        for l, q in enumerate(qs):
            assert w.set_base_q(l, q) == 0
        status = []

        def worker(k):
            for j in jobs[k::threads]:
                status.append(w.append_atom(j[0], j[1], j[2], j[3], j[4]))
        th = [threading.Thread(target=worker, args=(k,)) for k in range(threads)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        assert status == [0] * len(jobs)
        for l, az, ay, ax, _ in jobs[:20]:
            assert w.coverage(l, az, ay, ax) in (1, 2)
    data = open(path, "rb").read()
    a = vc.Archive(data)
    for lod, want in enumerate(g["lod_sha256"]):
        s, out = a.decode_lod(lod)
        assert s == 0 and hashlib.sha256(out.tobytes()).hexdigest() == want, lod
    ref = load_archive(g)
    assert abs(len(data) - len(ref)) < 16 * 32768 * 16   # same payloads, blocks in another order


def test_random_marks_sessions_match_reference(vc):
    """Random writer sessions of zero marks, base_q settings and coverage
    queries (odd and large dims, coordinates in and past every LOD, repeated
    and overlapping marks, q outside the clamp range), no atom contents, run
    live on the reference's own writer (oracle/_ref, built on this host only)
    and on this library: every op's result and the closed file's bytes are the
    reference's."""
    import refcodec
    if not refcodec.available():
        pytest.skip("reference build (oracle/_ref) not present on this host")
    R = W.bind(ctypes.CDLL(refcodec.REF_SO))   # own handle: the script's ctypes types
    L = mylib(vc)
    rng = np.random.default_rng(0x3A4C)
    for trial in range(24):
        dims = [int(rng.choice([1, 31, 32, 33, 97, 300, 1024, 2100, 4097])) for _ in range(3)]
        ops = [["create", dims, float(rng.choice([1.0, 12.0, 100.0]))]]
        for _ in range(int(rng.integers(5, 60))):
            lod = int(rng.choice([0, 0, 1, 2, 3, 7, 8, -1]))
            d = [max(1, (v + (1 << max(lod, 0)) - 1) >> max(lod, 0)) for v in dims]
            at = [int(rng.integers(0, (v + 31) // 32 + 2)) for v in d]   # x, y, z atoms, a few past the edge
            rg = [int(rng.integers(0, (v + 1023) // 1024 + 2)) for v in d]
            k = int(rng.integers(0, 10))
            if k < 4:
                ops.append(["zatom", lod, at[2], at[1], at[0]])
            elif k < 5:
                ops.append(["zregion", lod, rg[2], rg[1], rg[0]])
            elif k < 6:
                ops.append(["q", lod, float(rng.choice([0.001, 0.05, 1.5, 4096.0, 9000.0]))])
            else:
                ops.append(["cov", lod, at[2], at[1], at[0]])
        ops.append(["close"])
        s = {"volume": [[8, 8, 8], 1], "ops": ops}
        assert W.run(L, s, vc.synth) == W.run(R, s, vc.synth), trial
