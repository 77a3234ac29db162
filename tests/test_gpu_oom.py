"""Allocation failures. vcg_debug_fail_alloc(n) makes the n-th device or
pinned-host allocation of the library from now on fail (as cudaMalloc does
when the device is full). For each public call, the sweep lets the 1st, 2nd,
3rd ... allocation of a fresh call fail in turn, until a call makes fewer
allocations than n. A call that met the failure must not crash and must
return VC_ERR_OOM, or succeed with the right result where it has a path that
needs no new allocation (a pageable copy without its pinned ring, an encode
without its cached forward transform, a shared second stream). The run that
meets no failure must give the right result: the library stays usable after
every failure, and device memory does not leak.

Each call runs in a thread of its own, so its per-thread scratch buffers are
allocated afresh and every attempt sees the same sequence of allocations."""
import ctypes
import hashlib
import struct
import threading

import numpy as np
import pytest

from conftest import load_archive

pytestmark = pytest.mark.gpu

LIMIT = 96                # more allocations than any call here makes
LEAK_TOLERANCE = 64 << 20  # device bytes: allocation granularity, cached archive blocks


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


def in_thread(vc, fn):
    box = {}

    def body():
        try:
            box["r"] = fn()
        except BaseException as e:   # noqa: BLE001 - handed to the caller
            box["e"] = e
        box["err"] = vc.last_error()   # the error text is per thread

    t = threading.Thread(target=body)
    t.start()
    t.join()
    if "e" in box:
        raise box["e"]
    return box["r"], box["err"]


def sweep(vc, op, right):
    """op() -> (status, result); right(result) -> bool. Returns the number of
    allocations the call makes."""
    L = vc.lib()
    (s, r), err = in_thread(vc, op)   # warm: lazily loaded kernels, cached blocks
    assert s == vc.VC_OK and right(r), err
    _, free0, _ = vc.device_memory()
    bad = []
    for n in range(1, LIMIT + 1):
        L.vcg_debug_fail_alloc(n)
        try:
            (s, r), err = in_thread(vc, op)
        finally:
            hit = L.vcg_debug_fail_alloc(0) == -1
        if not hit:   # the call made fewer than n allocations: nothing failed
            assert not bad, bad
            assert s == vc.VC_OK and right(r), (n, s, err)
            _, free1, _ = vc.device_memory()
            assert free1 + LEAK_TOLERANCE >= free0, (free0, free1)
            return n - 1
        if s == vc.VC_OK:
            if not right(r):
                bad.append((n, "succeeded with a wrong result"))
        elif s != vc.VC_ERR_OOM:
            bad.append((n, s, err))
    pytest.fail(f"more than {LIMIT} allocations")


@pytest.fixture(scope="module")
def prime(golden):
    c = golden["synth_prime_97x131x65_t20"]
    return c, load_archive(c)


def test_encode(vc, gpu, prime):
    c, data = prime
    nx, ny, nz = c["dims"]
    vol = vc.synth(nx, ny, nz, c["seed"])
    assert sweep(vc, lambda: vc.encode(vol, c["target"]), lambda d: sha(d) == c["sha256"]) > 0


def test_encode_device(vc, gpu, prime):
    c, data = prime
    nx, ny, nz = c["dims"]
    dv = vc.DeviceBuffer(nx * ny * nz + 16)
    dv.upload(vc.synth(nx, ny, nz, c["seed"]))

    def op():
        s, d, _ = vc.encode_device(dv, (nx, ny, nz), c["target"])
        return s, d

    assert sweep(vc, op, lambda d: sha(d) == c["sha256"]) > 0
    dv.free()


def test_encode_with_pyramid_options(vc, gpu):
    vol = vc.synth(96, 80, 72, 0x0A110C)
    s, want = vc.encode_ds(vol, 10.0, vc.DS_CBOX, 0.25)
    assert s == vc.VC_OK
    assert sweep(vc, lambda: vc.encode_ds(vol, 10.0, vc.DS_CBOX, 0.25), lambda d: d == want) > 0


def _decode_lods(vc, data, nlod):
    a = vc.Archive(data)
    try:
        outs = []
        for lod in range(nlod):
            s, v = a.decode_lod(lod)
            if s:
                return s, None
            outs.append(sha(v))
        return vc.VC_OK, outs
    finally:
        a.close()


def test_decode_lod_to_host(vc, gpu, prime):
    c, data = prime
    nlod = len(c["lod_sha256"])
    assert sweep(vc, lambda: _decode_lods(vc, data, nlod), lambda r: r == c["lod_sha256"]) > 0


def test_decode_lod_to_device(vc, gpu, prime):
    c, data = prime
    nx, ny, nz = c["dims"]
    dbuf = vc.DeviceBuffer(nx * ny * nz)

    def op():
        a = vc.Archive(data)
        try:
            s = a.decode_lod_device(0, dbuf)
            return s, sha(dbuf.download()) if s == vc.VC_OK else None
        finally:
            a.close()

    assert sweep(vc, op, lambda h: h == c["lod_sha256"][0]) > 0
    dbuf.free()


@pytest.fixture(scope="module")
def big(vc, gpu):
    """A 512^3 archive: its LOD0 (128 MiB) takes the pipelined copy-out, and
    into pageable memory the pinned bounce ring."""
    dv = vc.synth_device(512, 512, 512, 0x0A110D)
    s, data, _ = vc.encode_device(dv, (512, 512, 512), 10.0)
    dv.free()
    assert s == vc.VC_OK
    a = vc.Archive(data)
    s, v = a.decode_lod(0)
    a.close()
    assert s == vc.VC_OK
    return data, sha(v)


@pytest.mark.parametrize("pinned", [False, True])
def test_large_decode_to_host(vc, gpu, big, pinned):
    data, want = big
    n = 512 ** 3
    if pinned:
        p = vc.lib().vcg_alloc_host(n)
        assert p
        out = np.ctypeslib.as_array((ctypes.c_uint8 * n).from_address(p)).reshape(512, 512, 512)
    else:
        out = np.zeros((512, 512, 512), np.uint8)

    def op():
        a = vc.Archive(data)
        try:
            out[:] = 0
            s, v = a.decode_lod(0, out)
            return s, sha(v) if s == vc.VC_OK else None
        finally:
            a.close()

    try:
        assert sweep(vc, op, lambda h: h == want) > 0
    finally:
        if pinned:
            vc.lib().vcg_free_host(p)


def _boxes():
    rng = np.random.default_rng(0x0A11)
    out = []
    for i in range(24):
        lod = i % 2
        hi = (97 >> lod, 131 >> lod, 65 >> lod)
        lo = [int(rng.integers(0, h - 1)) for h in hi]
        up = [int(rng.integers(l + 1, h + 1)) for l, h in zip(lo, hi)]
        out.append((lod, (lo[0], lo[1], lo[2], up[0], up[1], up[2])))
    return out


def _box_bytes(b):
    return (b[3] - b[0]) * (b[4] - b[1]) * (b[5] - b[2])


@pytest.fixture(scope="module")
def boxes(oracle, prime):
    c, data = prime
    o = oracle.Archive(data)
    reqs = _boxes()
    want = []
    for lod, b in reqs:
        s, v = o.decode_region(lod, b)
        assert s == 0
        want.append(sha(v))
    o.close()
    return reqs, want


def test_decode_region(vc, gpu, prime, boxes):
    c, data = prime
    reqs, want = boxes

    def op():
        a = vc.Archive(data)
        try:
            got = []
            for lod, b in reqs[:6]:
                s, v = a.decode_region(lod, b)
                if s:
                    return s, None
                got.append(sha(v))
            return vc.VC_OK, got
        finally:
            a.close()

    assert sweep(vc, op, lambda g: g == want[:6]) > 0


@pytest.mark.parametrize("on_device", [False, True])
def test_decode_regions_batched(vc, gpu, prime, boxes, on_device):
    c, data = prime
    reqs, want = boxes
    outs = [vc.DeviceBuffer(_box_bytes(b)) if on_device else np.zeros(_box_bytes(b), np.uint8) for _, b in reqs]

    def op():
        a = vc.Archive(data)
        try:
            s, st = a.decode_regions(reqs, outs, on_device)
            if s:
                return s, None
            if (np.asarray(st) != 0).any():
                return int(np.asarray(st)[np.asarray(st) != 0][0]), None
            return vc.VC_OK, [sha(o.download() if on_device else o) for o in outs]
        finally:
            a.close()

    assert sweep(vc, op, lambda g: g == want) > 0
    if on_device:
        for o in outs:
            o.free()


def test_served_regions(vc, gpu, prime, boxes):
    c, data = prime
    reqs, want = boxes
    outs = [np.zeros(_box_bytes(b), np.uint8) for _, b in reqs]

    def op():
        a = vc.Archive(data)
        try:
            with a.server(device_budget=64 << 20, max_batch=8, workers=2) as srv:
                tix = [srv.submit(lod, b, o) for (lod, b), o in zip(reqs, outs)]
                res = [srv.wait(t)[0] for t in tix]
            bad = [s for s in res if s != vc.VC_OK]
            return (bad[0] if bad else vc.VC_OK), [sha(o) for o in outs]
        finally:
            a.close()

    assert sweep(vc, op, lambda g: g == want) > 0


def test_streamed_regions(vc, gpu, prime, boxes):
    c, data = prime
    reqs, want = boxes

    def op():
        a = vc.StreamingArchive(data)
        try:
            got = []
            for lod, b in reqs[:6]:
                s, v = a.decode_region(lod, b)
                if s:
                    return s, None
                got.append(sha(v))
            return vc.VC_OK, got
        finally:
            a.close()

    assert sweep(vc, op, lambda g: g == want[:6]) > 0


def test_repack_v2(vc, gpu, prime):
    c, data = prime
    a = vc.Archive(data)
    s, want = a.repack_v2()
    a.close()
    assert s == vc.VC_OK

    def op():
        a = vc.Archive(data)
        try:
            return a.repack_v2()
        finally:
            a.close()

    assert sweep(vc, op, lambda d: d == want) > 0


def test_writer_session(vc, gpu, tmp_path):
    vol = vc.synth(64, 64, 64, 0x0A110E)
    atoms = [np.ascontiguousarray(vol[z * 32:z * 32 + 32, y * 32:y * 32 + 32, x * 32:x * 32 + 32])
             for z in range(2) for y in range(2) for x in range(2)]
    count = [0]

    def op():
        count[0] += 1
        path = str(tmp_path / f"w{count[0]}.vca")
        w = vc.Writer(path, (64, 64, 64), 10.0)
        if not w:
            return vc.VC_ERR_OOM, None
        s = w.set_base_q(0, 1.5)
        for i, v in enumerate(atoms[:4]):
            s = s or w.append_atom(0, i // 4, (i // 2) % 2, i % 2, v)
        for i, v in enumerate(atoms[4:], 4):
            s = s or w.append_atom_async(0, i // 4, (i // 2) % 2, i % 2, v)
        fs, failed = w.flush()
        s = s or fs
        s2, anyv, _ = w.decode_2x2x2(0, 0, 0, 0)
        w.close()
        if s or s2:
            return s or s2, None
        with open(path, "rb") as f:
            return vc.VC_OK, f.read()

    (s, want), err = in_thread(vc, op)
    assert s == vc.VC_OK, err
    assert sweep(vc, op, lambda d: d == want) > 0


def test_dct_and_downscale(vc, gpu, oracle):
    vol = vc.synth(64, 64, 64, 0x0A110F)
    dv = vc.DeviceBuffer(vol.size)
    dv.upload(vol)
    coef = vc.DeviceBuffer(vol.size * 4)
    back = vc.DeviceBuffer(vol.size)
    want_ds = oracle.ds_downscale2x(vol, vc.DS_BOX, 0.5)

    def op():
        s, _ = vc.dct_forward(dv, (64, 64, 64), 128, vc.DCT_BUTTERFLY, coef)
        if s:
            return s, None
        s, _ = vc.dct_inverse(coef, (64, 64, 64), 128, vc.DCT_BUTTERFLY, back)
        if s:
            return s, None
        s, ds = vc.downscale2x(vol, vc.DS_BOX)
        return s, (back.download(), ds)

    (s, (want_back, ds)), err = in_thread(vc, op)   # the transforms' parity is pinned elsewhere
    assert s == vc.VC_OK and np.array_equal(ds, want_ds), err
    assert sweep(vc, op, lambda r: np.array_equal(r[0], want_back) and np.array_equal(r[1], want_ds)) > 0
    for b in (dv, coef, back):
        b.free()


def test_failed_residency_is_retried(vc, gpu, prime):
    """An archive whose first upload ran out of memory becomes resident on a
    later call: the failure is not remembered."""
    c, data = prime
    L = vc.lib()

    def op():
        a = vc.Archive(data)
        try:
            L.vcg_debug_fail_alloc(1)
            try:
                s1 = a.make_resident()
            finally:
                hit = L.vcg_debug_fail_alloc(0) == -1
            s2, v = a.decode_lod(0)
            return s1, hit, s2, sha(v)
        finally:
            a.close()

    (s1, hit, s2, h), err = in_thread(vc, op)
    assert hit and s1 == vc.VC_ERR_OOM
    assert s2 == vc.VC_OK and h == c["lod_sha256"][0], err


def test_noalloc_decode_makes_no_allocation(vc, gpu, prime):
    """vcg_decode_atoms_noalloc never allocates: an armed failure stays armed."""
    c, data = prime
    a = vc.Archive(data)
    dev = vc.DeviceBuffer(len(data))
    dev.upload(np.frombuffer(data, np.uint8))
    cov, off, ln = a.payload_range(0, 0, 0, 0)
    offs, lens = np.array([off], np.uint64), np.array([ln], np.uint32)
    out = vc.DeviceBuffer(32768)
    L = vc.lib()
    q0 = struct.unpack_from("<f", data, 72)[0]
    assert L.vcg_decode_atoms_noalloc(dev.ptr, len(data), vc.ptr(offs), vc.ptr(lens), 1, q0, out.ptr) == vc.VC_OK
    L.vcg_debug_fail_alloc(1)
    try:
        s = L.vcg_decode_atoms_noalloc(dev.ptr, len(data), vc.ptr(offs), vc.ptr(lens), 1, q0, out.ptr)
    finally:
        left = L.vcg_debug_fail_alloc(0)
    assert s == vc.VC_OK and left == 1
    s, want = a.decode_atom(0, 0, 0, 0)
    assert np.array_equal(out.download(), want)
    for b in (dev, out):
        b.free()
    a.close()
