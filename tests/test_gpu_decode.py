"""GPU decode parity: every LOD, every atom and random regions of archives
produced by the reference, bit-exact against the golden hashes and the oracle;
malformed archives return the oracle's status and partial output."""
import hashlib
import threading

import numpy as np
import pytest

from conftest import load_archive

pytestmark = pytest.mark.gpu

STORED = ["synth_64_t10", "synth_prime_97x131x65_t20", "synth_flat_96x64x33_t100", "tiny_1x1x1"]


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


@pytest.mark.parametrize("name", STORED)
def test_decode_every_lod_atom_region(vc, gpu, golden, name):
    c = golden[name]
    a = vc.Archive(load_archive(c))
    nlod = len(c["lod_sha256"])
    for lod in range(nlod):
        s, vol = a.decode_lod(lod)
        assert s == 0 and sha(vol) == c["lod_sha256"][lod], lod
        _, (nx, ny, nz) = a.lod_dims(lod)
        h = hashlib.sha256()
        for az in range((nz + 31) // 32):
            for ay in range((ny + 31) // 32):
                for ax in range((nx + 31) // 32):
                    s, at = a.decode_atom(lod, ax, ay, az)
                    assert s == 0
                    h.update(at.tobytes())
        assert h.hexdigest() == c["atoms_sha256"][lod], lod
    for r in c["regions"]:
        s, out = a.decode_region(r["lod"], tuple(r["box"]))
        assert s == r["status"] and sha(out) == r["sha256"]


@pytest.mark.parametrize("name", ["ref_test_basic", "extreme_zero", "extreme_voxel", "extreme_line", "extreme_sat"])
def test_decode_reference_writer_archives(vc, gpu, golden, name):
    c = golden[name]
    a = vc.Archive(load_archive(c))
    nx, ny, nz = c["dims"]
    i = 0
    for az in range((nz + 31) // 32):
        for ay in range((ny + 31) // 32):
            for ax in range((nx + 31) // 32):
                s, at = a.decode_atom(0, ax, ay, az)
                assert s == 0 and sha(at) == c["atom_sha256"][i], (az, ay, ax)
                i += 1
    s, full = a.decode_lod(0)
    assert s == 0 and sha(full) == c["lod0_sha256"]


def test_random_regions_match_oracle(vc, oracle, gpu, golden):
    data = load_archive(golden["synth_prime_97x131x65_t20"])
    a, o = vc.Archive(data), oracle.Archive(data)
    rng = np.random.default_rng(7)
    for _ in range(150):
        lod = int(rng.integers(0, o.nlod))
        _, d = o.lod_dims(lod)
        lo = [int(rng.integers(0, d[k])) for k in range(3)]
        hi = [int(rng.integers(lo[k] + 1, d[k] + 1)) for k in range(3)]
        box = (lo[0], lo[1], lo[2], hi[0], hi[1], hi[2])
        s1, g = a.decode_region(lod, box)
        s2, r = o.decode_region(lod, box)
        assert s1 == s2 == 0 and (g == r).all(), (lod, box)


def test_device_output_matches_host_output(vc, gpu, golden):
    c = golden["synth_prime_97x131x65_t20"]
    a = vc.Archive(load_archive(c))
    s, (nx, ny, nz) = a.lod_dims(0)
    buf = vc.DeviceBuffer(nx * ny * nz)
    assert a.decode_lod_device(0, buf) == 0
    assert sha(buf.download()) == c["lod_sha256"][0]
    box = (5, 17, 3, 90, 100, 60)
    s, host = a.decode_region(0, box)
    assert a.decode_region_device(0, box, buf) == 0
    assert (buf.download(host.size) == host).all()


def test_concurrent_decodes_are_independent(vc, gpu, golden):
    c = golden["synth_64_t10"]
    a = vc.Archive(load_archive(c))
    results = {}

    def work(k):
        outs = []
        for _ in range(4):
            s, vol = a.decode_lod(0)
            outs.append((s, sha(vol)))
        results[k] = outs

    ts = [threading.Thread(target=work, args=(k,)) for k in range(4)]
    [t.start() for t in ts]
    [t.join() for t in ts]
    for k in range(4):
        assert all(r == (0, c["lod_sha256"][0]) for r in results[k])


def _slot_offset(data, lod, az, ay, ax):
    """File offset of an atom's L2 slot (v1 hash probe, src/vc/vc.c:1349-1402)."""
    import struct
    l1_cap, _, l1_off = struct.unpack_from("<QQQ", data, 40)

    def mix64(x):
        m = (1 << 64) - 1
        x = (x + 0x9E3779B97F4A7C15) & m
        x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & m
        x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & m
        return x ^ (x >> 31)

    key = (lod << 45) | ((az // 32) << 30) | ((ay // 32) << 15) | (ax // 32)
    i = mix64(key) & (l1_cap - 1)
    while True:
        k, b = struct.unpack_from("<QQ", data, l1_off + 16 * i)
        if k == key and b:
            break
        i = (i + 1) & (l1_cap - 1)
    return b + (((az % 32) * 32 + ay % 32) * 32 + ax % 32) * 16


@pytest.mark.parametrize("kind", ["len_past_end", "off_past_end", "len_zero", "off_wraps"])
def test_bad_slot_is_format_error_with_partial_output(vc, oracle, gpu, golden, kind):
    import struct
    data = bytearray(load_archive(golden["synth_prime_97x131x65_t20"]))
    so = _slot_offset(data, 0, 1, 2, 1)
    off, ln = struct.unpack_from("<QI", data, so)
    if kind == "len_past_end":
        struct.pack_into("<I", data, so + 8, len(data))
    elif kind == "off_past_end":
        struct.pack_into("<Q", data, so, len(data) + 10)
    elif kind == "len_zero":
        struct.pack_into("<I", data, so + 8, 0)
    else:
        struct.pack_into("<Q", data, so, (1 << 64) - 8)
    data = bytes(data)
    a, o = vc.Archive(data), oracle.Archive(data)
    box = (0, 0, 0, 97, 131, 65)
    g = np.full(97 * 131 * 65, 0xAB, np.uint8)
    r = g.copy()
    s1, _ = a.decode_region(0, box, g)
    s2, _ = o.decode_region(0, box, r)
    assert s1 == s2 == vc.VC_ERR_FORMAT
    assert (g == r).all()
    s1, at = a.decode_atom(0, 1, 2, 1)
    s2, at2 = o.decode_atom(0, 1, 2, 1)
    assert s1 == s2 == vc.VC_ERR_FORMAT and (at == 0).all() and (at2 == 0).all()


def test_corrupt_payloads_match_oracle(vc, oracle, gpu, golden):
    """Random bytes in the payload area: the GPU must decode exactly what the
    oracle decodes (or report the same malformed-stream error), never read
    outside the payload."""
    import struct
    base = bytearray(load_archive(golden["synth_64_t10"]))
    rng = np.random.default_rng(99)
    for trial in range(6):
        data = bytearray(base)
        for (az, ay, ax) in [(0, 0, 0), (1, 1, 0), (0, 1, 1)]:
            so = _slot_offset(data, 0, az, ay, ax)
            off, ln = struct.unpack_from("<QI", data, so)
            k = int(rng.integers(1, ln))
            data[off + k: off + ln] = rng.integers(0, 256, ln - k).astype(np.uint8).tobytes()
        data = bytes(data)
        a, o = vc.Archive(data), oracle.Archive(data)
        for lod in range(o.nlod):
            s1, g = a.decode_lod(lod)
            s2, r = o.decode_lod(lod)
            assert s1 == s2
            if s1 == 0:
                assert (g == r).all()


def test_truncated_archive_matches_oracle(vc, oracle, gpu, golden):
    data = load_archive(golden["synth_prime_97x131x65_t20"])
    for cut in [len(data) - 1, len(data) - 5000, 700000, 530000]:
        d = data[:cut]
        a, o = vc.Archive(d), oracle.Archive(d)
        assert bool(a) == bool(o.h)
        if not a:
            continue
        for lod in range(o.nlod):
            s1, g = a.decode_lod(lod)
            s2, r = o.decode_lod(lod)
            assert s1 == s2, (cut, lod)
            if s1 == 0:
                assert (g == r).all()


def test_large_decode_into_pinned_memory_overlaps_copy_out(vc, gpu):
    """A LOD0 decode of >= 64 MiB into pinned host memory takes the path that
    copies each transformed slab out while the next one is transformed; it must
    give the same bytes and statuses as the plain path into pageable memory,
    also when an atom in the middle of the volume is malformed (then only the
    atoms before it may be written)."""
    import ctypes
    import struct
    n = 512
    dv = vc.synth_device(n, n, n, vc.config_seed(2))
    s, data = vc.encode_q(dv, 10.0, [2.0 * 0.6 ** l for l in range(8)], on_device=(n, n, n))
    assert s == 0
    dv.free()
    L = vc.lib()
    pinned = L.vcg_alloc_host(n ** 3)
    assert pinned
    try:
        pv = (ctypes.c_uint8 * (n ** 3)).from_address(pinned)
        view = np.frombuffer(pv, np.uint8)
        bad = bytearray(data)
        so = _slot_offset(bad, 0, 8, 5, 9)   # atom (az, ay, ax) = (8, 5, 9): mid-volume
        struct.pack_into("<I", bad, so + 8, len(bad))
        for arc_bytes in (bytes(data), bytes(bad)):
            a = vc.Archive(arc_bytes)
            ref = np.full(n ** 3, 0x3C, np.uint8)
            s_ref, _ = a.decode_lod(0, ref.reshape(n, n, n))
            view[:] = 0x3C
            d = vc.Dims()
            s_pin = L.vc_decode_lod(a.h, 0, pinned, ctypes.byref(d))
            assert s_pin == s_ref
            assert np.array_equal(view, ref)
        assert s_ref == vc.VC_ERR_FORMAT
    finally:
        L.vcg_free_host(pinned)


def test_large_decode_into_pageable_memory(vc, gpu):
    """Outputs of >= 16 MiB in pageable memory are copied out through pinned
    32 MiB bounce chunks by host threads: the bytes equal a decode into device
    memory for whole chunks, a ragged last chunk and an output just below the
    threshold (one plain copy)."""
    n = 512
    dv = vc.synth_device(n, n, n, vc.config_seed(2))
    s, data = vc.encode_q(dv, 10.0, [2.0 * 0.6 ** l for l in range(8)], on_device=(n, n, n))
    assert s == 0
    dv.free()
    a = vc.Archive(data)
    for box in [(0, 0, 0, n, n, n), (3, 5, 7, 509, 487, 311), (0, 0, 0, 256, 256, 255)]:
        nb = (box[3] - box[0]) * (box[4] - box[1]) * (box[5] - box[2])
        host = np.full(nb, 0x77, np.uint8)
        st, _ = a.decode_region(0, box, host)
        assert st == vc.VC_OK
        dbuf = vc.DeviceBuffer(nb)
        assert a.decode_region_device(0, box, dbuf) == vc.VC_OK
        assert np.array_equal(host, dbuf.download(nb)), box
        dbuf.free()


@pytest.mark.gpu
def test_latency_decoder_streams_staged_and_not(vc, oracle, gpu):
    """Boxes of a few atoms take the latency decoder, which stages an atom's
    stream in 40 KiB of shared memory and reads longer streams from global
    memory: a noise volume coded at the smallest q has streams on both sides of
    that limit; every atom, and a box of them, must equal the oracle."""
    vol = np.random.default_rng(0x1A7).integers(0, 256, (64, 64, 96)).astype(np.uint8)
    vol[:, :, 64:] //= 16   # a quieter third: shorter streams
    s, data = vc.encode_q(vol, 1.0, [0.05] * 8)
    assert s == 0
    a, o = vc.Archive(data), oracle.Archive(data)
    lens = []
    for az in range(2):
        for ay in range(2):
            for ax in range(3):
                lens.append(a.payload_range(0, az, ay, ax)[2])
                s1, g = a.decode_atom(0, ax, ay, az)
                s2, r = o.decode_atom(0, ax, ay, az)
                assert s1 == s2 == 0 and np.array_equal(g, r), (az, ay, ax)
    assert min(lens) < 40 * 1024 <= max(lens), lens
    box = (0, 0, 0, 96, 64, 64)
    s1, g = a.decode_region(0, box)
    s2, r = o.decode_region(0, box)
    assert s1 == s2 == 0 and np.array_equal(g, r)
