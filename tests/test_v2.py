"""The v2 container (src/vc/vc.c:706-718; region directory + region-contiguous
blobs). Fixtures are the stored v1 golden archives rewritten by the reference's
own repack tool (tests/golden/gen_v2.py). Host-side reading (header, directory,
coverage, payload ranges) and the C oracle run on the CPU; decode parity and the
device repack (byte-identical to the reference tool) run on the GPU."""
import hashlib
import json
import lzma
import os
import struct

import numpy as np
import pytest

import oraclelib as O
from conftest import GOLDEN, load_archive

V2 = json.load(open(os.path.join(GOLDEN, "v2.json")))["cases"]
IDS = [c["name"] for c in V2]


def load_v2(case):
    return lzma.decompress(open(os.path.join(GOLDEN, case["file"]), "rb").read())


def v1_of(golden, case):
    return load_archive(golden[case["name"]])


def atoms_of(dims):
    nx, ny, nz = dims
    for az in range((nz + 31) // 32):
        for ay in range((ny + 31) // 32):
            for ax in range((nx + 31) // 32):
                yield az, ay, ax


@pytest.mark.parametrize("case", V2, ids=IDS)
def test_fixture_is_v2(case):
    data = load_v2(case)
    assert hashlib.sha256(data).hexdigest() == case["sha256"]
    magic, ver = struct.unpack_from("<II", data, 0)
    dir_off, cnt, total = struct.unpack_from("<QQQ", data, 40)
    assert magic == 0x00314356 and ver == 2 and dir_off == 128 and total == len(data)


@pytest.mark.parametrize("case", V2, ids=IDS)
def test_host_reader_v2_matches_v1(vc, golden, case):
    """Coverage and payload bytes of every atom read through the v2 directory
    equal those of the v1 index (no GPU needed)."""
    v1, v2 = v1_of(golden, case), load_v2(case)
    a1, a2 = vc.Archive(v1), vc.Archive(v2)
    assert a1.version() == 1 and a2.version() == 2
    nlod = struct.unpack_from("<I", v1, 20)[0]
    for lod in range(nlod):
        s, dims = a1.lod_dims(lod)
        assert a2.lod_dims(lod) == (s, dims)
        for az, ay, ax in atoms_of(dims):
            c1, o1, l1 = a1.payload_range(lod, az, ay, ax)
            c2, o2, l2 = a2.payload_range(lod, az, ay, ax)
            assert c1 == c2 and l1 == l2, (lod, az, ay, ax)
            if c1 == vc.VC_PRESENT:
                assert v1[o1:o1 + l1] == v2[o2:o2 + l2]


@pytest.mark.parametrize("case", V2, ids=IDS)
def test_oracle_decodes_v2_like_v1(golden, case):
    v1, v2 = v1_of(golden, case), load_v2(case)
    o1, o2 = O.Archive(v1), O.Archive(v2)
    assert O.lib().orc_archive_version(o2.h) == 2
    for lod in range(o1.nlod):
        s1, d1 = o1.decode_lod(lod)
        s2, d2 = o2.decode_lod(lod)
        assert s1 == s2 and np.array_equal(d1, d2), lod


@pytest.mark.parametrize("case", V2, ids=IDS)
def test_reference_decodes_v2_like_v1(golden, case):
    """Pins the v2 fixtures with the reference's own reader (where it is built)."""
    ref_so = os.path.join(os.path.dirname(GOLDEN), "..", "oracle", "_ref", "libvcref.so")
    if not os.path.exists(ref_so):
        pytest.skip("reference build not present")
    import refcodec
    v1, v2 = v1_of(golden, case), load_v2(case)
    r1, r2 = refcodec.RefArchive(v1), refcodec.RefArchive(v2)
    o = O.Archive(v1)
    for lod in range(o.nlod):
        s1, d1 = r1.decode_lod(lod)
        s2, d2 = r2.decode_lod(lod)
        assert s1 == s2 and np.array_equal(d1, d2), lod


@pytest.mark.gpu
@pytest.mark.parametrize("case", V2, ids=IDS)
def test_gpu_decodes_v2_like_v1_and_repacks_like_reference(vc, gpu, golden, case):
    v1, v2 = v1_of(golden, case), load_v2(case)
    a1, a2 = vc.Archive(v1), vc.Archive(v2)
    nlod = struct.unpack_from("<I", v1, 20)[0]
    for lod in range(nlod):
        s1, d1 = a1.decode_lod(lod)
        s2, d2 = a2.decode_lod(lod)
        assert s1 == s2 and np.array_equal(d1, d2), lod
    s, out = a1.repack_v2()
    assert s == vc.VC_OK
    assert len(out) == case["len"] and hashlib.sha256(out).hexdigest() == case["sha256"]
    s, out2 = a2.repack_v2()   # a v2 input gives the same image
    assert s == vc.VC_OK and out2 == out


@pytest.mark.gpu
def test_repack_refuses_bad_payload_range(vc, gpu, golden):
    from test_gpu_decode import _slot_offset
    data = bytearray(load_archive(golden["synth_prime_97x131x65_t20"]))
    so = _slot_offset(data, 0, 1, 2, 1)
    struct.pack_into("<I", data, so + 8, len(data))
    s, out = vc.Archive(bytes(data)).repack_v2()
    assert s == vc.VC_ERR_FORMAT and out is None
