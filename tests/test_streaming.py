"""Streaming archives (vc_open_streaming, src/vc/vc.c:1262-1280, 1329-1338;
the reference's tests/test_streaming.c and the v2 part of tests/test_repack.c).

A streaming archive pulls the header, index entries, slots and payloads
through a read callback. Results must equal those of the same bytes opened
flat. A read that fails makes an index entry or slot absent, and makes a
payload a VC_ERR_FORMAT of its atom. The poisoned byte source below fails
every read that overlaps a chosen byte range. It is applied to the reference
itself (where it is built), to the oracle's streaming mode, and to this
library: host-side lookups on the CPU, decodes on the GPU."""
import hashlib
import json
import lzma
import os
import struct

import numpy as np
import pytest

import oraclelib as O
from conftest import GOLDEN, load_archive

V2 = {c["name"]: c for c in json.load(open(os.path.join(GOLDEN, "v2.json")))["cases"]}
CASES = ["synth_prime_97x131x65_t20", "synth_64_t10", "extreme_line", "synth_flat_96x64x33_t100"]


def archive_bytes(golden, name, ver):
    if ver == 1:
        return load_archive(golden[name])
    return lzma.decompress(open(os.path.join(GOLDEN, V2[name]["file"]), "rb").read())


class Poisoned:
    """Byte source over `data` whose reads fail where they overlap a poisoned range."""

    def __init__(self, data, ranges=()):
        self.data, self.ranges, self.calls = bytes(data), list(ranges), 0

    def __call__(self, off, n):
        self.calls += 1
        if off + n > len(self.data):
            return None
        for lo, hi in self.ranges:
            if off < hi and lo < off + n:
                return None
        return self.data[off:off + n]


def atoms(dims):
    nx, ny, nz = dims
    for az in range((nz + 31) // 32):
        for ay in range((ny + 31) // 32):
            for ax in range((nx + 31) // 32):
                yield az, ay, ax


def slot_offset(data, lod, az, ay, ax):
    """File offset of an atom's 16-byte slot, v1 (hash probe) or v2 (directory)."""
    ver, nlod = struct.unpack_from("<I", data, 4)[0], struct.unpack_from("<I", data, 20)[0]
    si = (((az % 32) * 32 + ay % 32) * 32 + ax % 32) * 16
    if ver == 1:
        from test_gpu_decode import _slot_offset
        return _slot_offset(data, lod, az, ay, ax)
    return struct.unpack_from("<Q", data, dir_entry(data, lod, az // 32, ay // 32, ax // 32))[0] + si


def dir_entry(data, lod, rz, ry, rx):
    nx, ny, nz = struct.unpack_from("<III", data, 24)
    nlod = struct.unpack_from("<I", data, 20)[0]
    dir_off = struct.unpack_from("<Q", data, 40)[0]
    ri = 0
    for l in range(nlod):
        dx, dy, dz = [max(1, (v + (1 << l) - 1) >> l) for v in (nx, ny, nz)]
        grid = [((v + 31) // 32 + 31) // 32 for v in (dx, dy, dz)]
        if l == lod:
            return dir_off + 16 * (ri + (rz * grid[1] + ry) * grid[0] + rx)
        ri += grid[0] * grid[1] * grid[2]
    raise ValueError(lod)


def l1_bucket(data, lod, rz, ry, rx):
    """v1: file offset of a region's L1 bucket."""
    from test_gpu_decode import _slot_offset
    l1_cap, _, l1_off = struct.unpack_from("<QQQ", data, 40)
    blk = _slot_offset(data, lod, rz * 32, ry * 32, rx * 32) - 0
    for i in range(l1_cap):
        k, b = struct.unpack_from("<QQ", data, l1_off + 16 * i)
        if b and blk >= b and blk < b + 32768 * 16 and k == (lod << 45) | (rz << 30) | (ry << 15) | rx:
            return l1_off + 16 * i
    raise ValueError("region not indexed")


def poison_plan(data):
    """Ranges that poison one payload, one slot and one region index entry."""
    o = O.Archive(data)
    present = []
    for lod in range(o.nlod):
        _, dims = o.lod_dims(lod)
        for az, ay, ax in atoms(dims):
            c, off, ln = o.payload_range(lod, az, ay, ax)
            if c == 2:
                present.append((lod, az, ay, ax, off, ln))
    o.close()
    ranges = []
    if len(present) >= 1:   # a payload byte of the first present atom of LOD 0
        lod, az, ay, ax, off, ln = present[0]
        ranges.append((off + ln // 2, off + ln // 2 + 1))
    if len(present) >= 3:   # the slot of the third
        lod, az, ay, ax, _, _ = present[2]
        so = slot_offset(data, lod, az, ay, ax)
        ranges.append((so + 12, so + 13))
    coarse = [p for p in present if p[0] >= 1]
    if coarse:              # the index entry of a coarse LOD's region
        lod, az, ay, ax, _, _ = coarse[0]
        ver = struct.unpack_from("<I", data, 4)[0]
        e = dir_entry(data, lod, az // 32, ay // 32, ax // 32) if ver == 2 else \
            l1_bucket(data, lod, az // 32, ay // 32, ax // 32)
        ranges.append((e + 3, e + 4))
    return ranges


def every_outcome(arc, nlod, dims_of, decode_atoms=True):
    """Coverage, atom decodes and whole-LOD region decodes of an archive wrapper."""
    res = []
    for lod in range(nlod):
        _, dims = dims_of(lod)
        for az, ay, ax in atoms(dims):
            res.append(("cov", lod, az, ay, ax, arc.coverage(lod, az, ay, ax)))
            if decode_atoms:
                s, out = arc.decode_atom(lod, ax, ay, az)
                res.append(("atom", lod, az, ay, ax, s, hashlib.sha256(out.tobytes()).hexdigest()))
        nx, ny, nz = dims
        s, out = arc.decode_region(lod, (0, 0, 0, nx, ny, nz))
        res.append(("lod", lod, s, hashlib.sha256(out.tobytes()).hexdigest()))
    return res


class OracleView:
    """Uniform coverage / decode view of an oracle archive."""

    def __init__(self, a):
        self.a = a

    def coverage(self, lod, az, ay, ax):
        return O.lib().orc_atom_coverage(self.a.h, lod, az, ay, ax)

    def decode_atom(self, lod, ax, ay, az):
        return self.a.decode_atom(lod, ax, ay, az)

    def decode_region(self, lod, box):
        return self.a.decode_region(lod, box)


def oracle_outcome(data, ranges, decode_atoms=True):
    src = Poisoned(data, ranges)
    a = O.StreamingArchive(src, len(data))
    assert a.h
    try:
        return every_outcome(OracleView(a), a.nlod, a.lod_dims, decode_atoms)
    finally:
        a.close()


# ----------------------------------------------------------------------------- CPU

@pytest.mark.parametrize("ver", [1, 2])
@pytest.mark.parametrize("name", CASES)
def test_oracle_streaming_equals_flat(golden, name, ver):
    data = archive_bytes(golden, name, ver)
    flat = O.Archive(data)
    want = every_outcome(OracleView(flat), flat.nlod, flat.lod_dims)
    assert oracle_outcome(data, []) == want


@pytest.mark.parametrize("ver", [1, 2])
@pytest.mark.parametrize("name", CASES[:2])
def test_oracle_streaming_matches_reference_under_failed_reads(golden, name, ver):
    """Pins the oracle's streaming semantics to the reference's own reader."""
    import refcodec
    if not refcodec.available():
        pytest.skip("reference build not present")
    data = archive_bytes(golden, name, ver)
    ranges = poison_plan(data)
    assert len(ranges) == 3
    r = refcodec.RefStreamingArchive(Poisoned(data, ranges), len(data))
    assert r.h
    nlod = struct.unpack_from("<I", data, 20)[0]
    got = every_outcome(r, nlod, r.lod_dims)
    r.close()
    want = oracle_outcome(data, ranges)
    assert got == want
    # the poison shows: a FORMAT atom, and fewer present atoms than the flat archive has
    assert any(x[0] == "atom" and x[5] == 1 for x in want)


def test_open_streaming_rejects(vc, golden):
    data = archive_bytes(golden, "synth_64_t10", 1)
    assert not vc.StreamingArchive(Poisoned(data, [(0, 1)]), len(data))   # header read fails
    assert not vc.StreamingArchive(Poisoned(data), 100)                    # shorter than a header
    assert not vc.StreamingArchive(Poisoned(b"\0" * 256), 256)             # not an archive
    assert vc.lib().vc_open_streaming(None, None, len(data)) is None


@pytest.mark.parametrize("ver", [1, 2])
@pytest.mark.parametrize("name", CASES)
def test_host_lookups_streaming(vc, golden, name, ver):
    """Coverage, payload ranges and v2 blob ranges through the callback, clean
    and poisoned, equal the oracle's (host code only, no decode)."""
    data = archive_bytes(golden, name, ver)
    for ranges in ([], poison_plan(data)):
        src = Poisoned(data, ranges)
        a = vc.StreamingArchive(src, len(data))
        o = O.StreamingArchive(Poisoned(data, ranges), len(data))
        assert a and o.h and a.version() == ver
        for lod in range(o.nlod):
            s, dims = a.lod_dims(lod)
            assert (s, dims) == o.lod_dims(lod)
            for az, ay, ax in atoms(dims):
                assert a.payload_range(lod, az, ay, ax) == o.payload_range(lod, az, ay, ax), (lod, az, ay, ax)
        assert src.calls > 0
        if ver == 2 and not ranges:
            f = vc.Archive(data)
            for lod in range(o.nlod):
                _, dims = a.lod_dims(lod)
                for rz in range(((dims[2] + 31) // 32 + 31) // 32):
                    for ry in range(((dims[1] + 31) // 32 + 31) // 32):
                        for rx in range(((dims[0] + 31) // 32 + 31) // 32):
                            assert blob(vc, a, lod, rz, ry, rx) == blob(vc, f, lod, rz, ry, rx)
        a.close()
        o.close()


@pytest.mark.parametrize("ver", [1, 2])
def test_host_lookups_streaming_random_failed_reads(vc, golden, ver):
    """Reads failing over random byte ranges (1 to 5 ranges of 1 to 64 bytes,
    anywhere in the file: header, index, slots or payloads): the library's
    streaming archive opens exactly when the oracle's does and resolves every
    atom to the same payload range (host code only, no decode). Where the
    reference's own build exists, its streaming reader opens the same archives
    and gives every atom the oracle's coverage."""
    import refcodec
    with_ref = refcodec.available()
    rng = np.random.default_rng(0x57E + ver)
    opened = differs = 0
    for name in CASES:
        data = archive_bytes(golden, name, ver)
        clean = O.StreamingArchive(Poisoned(data), len(data))
        ref = {(lod, a): clean.payload_range(lod, *a) for lod in range(clean.nlod)
               for a in atoms(clean.lod_dims(lod)[1])}
        clean.close()
        keys = sorted(k for k, v in ref.items() if v[0] == 2)   # PRESENT atoms: their regions are indexed
        for _ in range(12):
            ranges = []
            for _ in range(int(rng.integers(1, 6))):
                if rng.integers(0, 2):   # anywhere
                    lo = int(rng.integers(0, len(data)))
                    ranges.append((lo, lo + int(rng.integers(1, 65))))
                    continue
                lod, (az, ay, ax) = keys[int(rng.integers(0, len(keys)))]   # a used slot or index entry
                if rng.integers(0, 2):
                    lo = slot_offset(data, lod, az, ay, ax) + int(rng.integers(0, 16))
                elif ver == 1:
                    lo = l1_bucket(data, lod, az // 32, ay // 32, ax // 32) + int(rng.integers(0, 16))
                else:
                    lo = dir_entry(data, lod, az // 32, ay // 32, ax // 32) + int(rng.integers(0, 16))
                ranges.append((lo, lo + 1))
            a = vc.StreamingArchive(Poisoned(data, ranges), len(data))
            o = O.StreamingArchive(Poisoned(data, ranges), len(data))
            assert bool(a) == bool(o.h), (name, ranges)
            if with_ref:
                r = refcodec.RefStreamingArchive(Poisoned(data, ranges), len(data))
                assert bool(r.h) == bool(o.h), ("oracle against the reference", name, ranges)
                for lod in range(o.nlod if o.h else 0):
                    for at in atoms(o.lod_dims(lod)[1]):
                        assert r.coverage(lod, *at) == o.coverage(lod, *at), ("oracle against the reference", lod, at)
                r.close()
            if not a:
                continue
            opened += 1
            for lod in range(o.nlod):
                s, dims = a.lod_dims(lod)
                assert (s, dims) == o.lod_dims(lod)
                for at in atoms(dims):
                    pr = a.payload_range(lod, *at)
                    assert pr == o.payload_range(lod, *at), (name, ranges, lod, at)
                    differs += pr != ref[(lod, at)]
            a.close()
            o.close()
    assert opened >= 20 and differs > 0


def blob(vc, a, lod, rz, ry, rx):
    import ctypes
    off, ln = ctypes.c_uint64(), ctypes.c_uint64()
    c = vc.lib().vc_region_blob_range(a.h, lod, rz, ry, rx, ctypes.byref(off), ctypes.byref(ln))
    return c, off.value, ln.value


def test_memory_source_counts(vc, golden):
    data = archive_bytes(golden, "synth_64_t10", 1)
    a = vc.StreamingArchive(data)
    assert a and a.reads()[0] == 1 and a.reads()[1] == 128   # the header
    a.coverage(0, 0, 0, 0)
    assert a.reads()[0] > 1


# ----------------------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("threads", [1, 4])
@pytest.mark.parametrize("ver", [1, 2])
@pytest.mark.parametrize("name", CASES + ["cfg1_256_t10"])
def test_gpu_streamed_decode_equals_golden(vc, gpu, golden, name, ver, threads):
    if ver == 2 and name not in V2:
        pytest.skip("no v2 fixture")
    g = golden[name]
    if "file" in g or ver == 2:
        data = archive_bytes(golden, name, ver)
    else:   # made by encoding the seeded volume; the fixture holds its SHA-256
        nx, ny, nz = g["dims"]
        dbuf = vc.synth_device(nx, ny, nz, g["seed"])
        s, data, _ = vc.encode_device(dbuf, (nx, ny, nz), g["target"])
        dbuf.free()
        assert s == vc.VC_OK and hashlib.sha256(data).hexdigest() == g["sha256"]
    prev = vc.set_stream_threads(threads)
    try:
        a = vc.StreamingArchive(data)
        for lod, want in enumerate(g.get("lod_sha256") or [g["lod0_sha256"]]):
            s, out = a.decode_lod(lod)
            assert s == vc.VC_OK and hashlib.sha256(out.tobytes()).hexdigest() == want, lod
        calls, nbytes = a.reads()
        assert calls > 1 and nbytes < 2 * len(data)   # pulled what it needed, not the archive many times over
        a.close()
    finally:
        vc.set_stream_threads(prev)


@pytest.mark.gpu
@pytest.mark.parametrize("threads", [1, 3])
@pytest.mark.parametrize("ver", [1, 2])
@pytest.mark.parametrize("name", CASES)
def test_gpu_streamed_failed_reads_match_oracle(vc, gpu, golden, name, ver, threads):
    """Poisoned payload, slot and index reads: every coverage, atom decode and
    whole-LOD decode (status and bytes) equals the oracle's streaming reader."""
    data = archive_bytes(golden, name, ver)
    ranges = poison_plan(data)
    want = oracle_outcome(data, ranges)
    prev = vc.set_stream_threads(threads)
    try:
        a = vc.StreamingArchive(Poisoned(data, ranges), len(data))
        nlod = struct.unpack_from("<I", data, 20)[0]
        got = every_outcome(a, nlod, a.lod_dims)
        a.close()
    finally:
        vc.set_stream_threads(prev)
    assert got == want


@pytest.mark.gpu
def test_gpu_streamed_regions_and_device_output(vc, gpu, golden):
    data = archive_bytes(golden, "synth_prime_97x131x65_t20", 1)
    flat, st = vc.Archive(data), vc.StreamingArchive(data)
    rng = np.random.default_rng(5)
    _, (nx, ny, nz) = flat.lod_dims(0)
    for _ in range(40):
        x0, y0, z0 = int(rng.integers(0, nx)), int(rng.integers(0, ny)), int(rng.integers(0, nz))
        box = (x0, y0, z0, int(rng.integers(x0 + 1, nx + 1)), int(rng.integers(y0 + 1, ny + 1)),
               int(rng.integers(z0 + 1, nz + 1)))
        s1, o1 = flat.decode_region(0, box)
        s2, o2 = st.decode_region(0, box)
        assert s1 == s2 == vc.VC_OK and np.array_equal(o1, o2), box
    buf = vc.DeviceBuffer(nx * ny * nz)
    assert st.decode_lod_device(0, buf) == vc.VC_OK
    assert np.array_equal(buf.download(nx * ny * nz), flat.decode_lod(0)[1].ravel())
    buf.free()


@pytest.mark.gpu
def test_gpu_streaming_made_resident(vc, gpu, golden):
    """vcg_make_resident pulls a streaming archive whole; batched decode and
    repack then work on it as on the flat archive."""
    data = archive_bytes(golden, "synth_prime_97x131x65_t20", 1)
    st = vc.StreamingArchive(data)
    assert st.make_resident() == vc.VC_OK
    assert st.reads()[1] >= len(data)
    s, v2 = st.repack_v2()
    assert s == vc.VC_OK and hashlib.sha256(v2).hexdigest() == V2["synth_prime_97x131x65_t20"]["sha256"]
    _, (nx, ny, nz) = st.lod_dims(0)
    box = (0, 0, 0, nx, ny, nz)
    outs = [np.zeros(nx * ny * nz, np.uint8)]
    s, stv = st.decode_regions([(0, box)], outs)
    assert s == vc.VC_OK and stv[0] == vc.VC_OK
    assert np.array_equal(outs[0], vc.Archive(data).decode_lod(0)[1].ravel())
    # a failed pull leaves the archive streaming and decodable
    bad = vc.StreamingArchive(Poisoned(data, [(len(data) - 1, len(data))]), len(data))
    assert bad.make_resident() == vc.VC_ERR_IO
    s, out = bad.decode_atom(0, 0, 0, 0)
    assert s == vc.VC_OK
