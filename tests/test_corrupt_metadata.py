"""Archive resolution on damaged metadata, without a GPU: the library's host
reader (header, v1 region hash table with its bounded probe, L2 slots and
their guards, v2 region directory; src/vc/vc.c:1285-1402) against the
oracle's, on golden archives with random bytes written into the L1 table, L1
block references replaced (empty, zero, claimed, misaligned, past the end,
into another table entry), random slot bytes, region keys overwritten, header
counters changed, v2 headers and directories hit, and truncations. Every
archive must open or fail to open on both, and then give the same LOD
dimensions and, for every atom (and one past each edge), the same coverage and
payload range. Where the reference's own build exists (oracle/_ref, this host
only) the oracle's answers are also checked against the reference's reader
on the same damaged archives, which pins the oracle there."""
import json
import lzma
import os
import struct

import numpy as np
import pytest

from conftest import GOLDEN, load_archive

V1 = ("synth_64_t10", "synth_prime_97x131x65_t20", "ref_test_basic", "synth_flat_96x64x33_t100")


def atom_table(o):
    out = []
    for lod in range(o.nlod):
        s, (nx, ny, nz) = o.lod_dims(lod)
        for az in range((nz + 31) // 32):
            for ay in range((ny + 31) // 32):
                for ax in range((nx + 31) // 32):
                    out.append((o.coverage(lod, az, ay, ax), o.payload_range(lod, az, ay, ax)))
    return out


def mismatch(vc, oracle, data):
    a, o = vc.Archive(data), oracle.Archive(data)
    if not a or not o.h:
        return None if bool(a) == bool(o.h) else ("open", bool(a), bool(o.h))
    if a.version() != oracle.lib().orc_archive_version(o.h):
        return ("version",)
    for lod in range(o.nlod + 1):
        if a.lod_dims(lod) != o.lod_dims(lod):
            return ("dims", lod)
        s, (nx, ny, nz) = o.lod_dims(lod)
        if s:
            continue
        for az in range((nz + 31) // 32 + 1):
            for ay in range((ny + 31) // 32 + 1):
                for ax in range((nx + 31) // 32 + 1):
                    c1, c2 = a.coverage(lod, az, ay, ax), o.coverage(lod, az, ay, ax)
                    p1, p2 = a.payload_range(lod, az, ay, ax), o.payload_range(lod, az, ay, ax)
                    if c1 != c2 or p1 != p2:
                        return ("atom", lod, az, ay, ax, c1, c2, p1, p2)
    return None


def reference_mismatch(oracle, data):
    """The oracle against the reference's reader (None: same answers)."""
    import ctypes
    import refcodec
    L = refcodec.lib()
    L.vc_atom_payload_range.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32,
                                        ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint64),
                                        ctypes.POINTER(ctypes.c_uint32)]
    o, r = oracle.Archive(data), refcodec.RefArchive(data)
    try:
        if bool(o.h) != bool(r.h):
            return ("open", bool(o.h), bool(r.h))
        if not o.h:
            return None
        for lod in range(o.nlod + 1):
            s, (nx, ny, nz) = o.lod_dims(lod)
            if r.lod_dims(lod) != (s, (nx, ny, nz)):
                return ("dims", lod)
            if s:
                continue
            for az in range((nz + 31) // 32 + 1):
                for ay in range((ny + 31) // 32 + 1):
                    for ax in range((nx + 31) // 32 + 1):
                        off, ln = ctypes.c_uint64(), ctypes.c_uint32()
                        c = L.vc_atom_payload_range(r.h, lod, az, ay, ax, ctypes.byref(off), ctypes.byref(ln))
                        if (o.coverage(lod, az, ay, ax) != r.coverage(lod, az, ay, ax) or
                                o.payload_range(lod, az, ay, ax) != (c, off.value, ln.value)):
                            return ("atom", lod, az, ay, ax)
        return None
    finally:
        o.close()
        r.close()


def corrupt_v1(rng, base, trial):
    l1_cap, _, l1_off = struct.unpack_from("<QQQ", base, 40)
    d = bytearray(base)
    kind = trial % 6
    if kind == 0:   # random bytes in the L1 table
        for _ in range(int(rng.integers(1, 8))):
            d[int(l1_off + rng.integers(0, 16 * l1_cap))] = int(rng.integers(0, 256))
    elif kind == 1:   # one L1 block reference replaced
        e = int(rng.integers(0, l1_cap))
        ref = int(rng.choice([0, 1, 2, 3, len(d) - 100, len(d) + 4096, int(rng.integers(0, 1 << 40)),
                              128 + 16 * int(rng.integers(0, l1_cap))]))
        struct.pack_into("<Q", d, l1_off + 16 * e + 8, ref)
    elif kind == 2:   # random bytes in the L2 blocks (slots) and payloads
        for _ in range(int(rng.integers(1, 20))):
            d[int(rng.integers(l1_off + 16 * l1_cap, len(d)))] = int(rng.integers(0, 256))
    elif kind == 3:
        d = d[:int(rng.integers(128, len(d)))]
    elif kind == 4:   # region keys overwritten
        for _ in range(3):
            struct.pack_into("<Q", d, l1_off + 16 * int(rng.integers(0, l1_cap)), int(rng.integers(0, 1 << 62)))
    else:   # L1 count and cursor
        struct.pack_into("<Q", d, 48, int(rng.integers(0, 2 * l1_cap + 2)))
        struct.pack_into("<Q", d, 64, int(rng.integers(0, len(d) * 2)))
    return bytes(d)


def corrupt_v2(rng, base, trial):
    d = bytearray(base)
    if trial % 3 == 2:
        return bytes(d[:int(rng.integers(128, len(d)))])
    hi = min(len(d), 128 + (1 << 16)) if trial % 3 == 0 else len(d)
    for _ in range(int(rng.integers(1, 10))):
        d[int(rng.integers(72 if trial % 5 == 0 else 104, hi))] = int(rng.integers(0, 256))
    return bytes(d)


@pytest.mark.parametrize("seed", [1, 2])
def test_damaged_metadata_resolves_like_oracle(vc, oracle, golden, seed):
    import refcodec
    with_ref = refcodec.available()
    rng = np.random.default_rng(seed)
    cases = [(load_archive(golden[n]), corrupt_v1, 60) for n in V1]
    for c in json.load(open(os.path.join(GOLDEN, "v2.json")))["cases"]:
        cases.append((lzma.decompress(open(os.path.join(GOLDEN, c["file"]), "rb").read()), corrupt_v2, 40))
    n = changed = 0
    for base, corrupt, trials in cases:
        o = oracle.Archive(base)
        clean = atom_table(o)
        o.close()
        for trial in range(trials):
            d = corrupt(rng, base, trial)
            bad = mismatch(vc, oracle, d)
            assert bad is None, (trial, bad)
            if with_ref:
                bad = reference_mismatch(oracle, d)
                assert bad is None, ("oracle against the reference", trial, bad)
            o = oracle.Archive(d)
            changed += not o.h or atom_table(o) != clean
            n += 1
    assert n == sum(t for _, _, t in cases) >= 500
    assert changed > n // 5   # the damage reaches the atoms' resolution, not only unused bytes
