"""Range-decoder policy 0 (no atom gets a warp of its own): decodes of up to
608 atoms (one per SM sub-partition: all the stored golden archives) run the
warp-lockstep decoder, several atoms per warp walking the scan positions
together; larger ones run the per-lane decoder (every lane of a warp its own
atom, atoms ordered by payload length), which the full-size archives of
test_gpu_encode exercise and the host build of test_host_decoders checks
stream by stream. Here the lockstep decoder must give the reference's bits on
the stored golden archives, and the oracle's statuses and bytes on corrupt and
truncated ones, including a stream with an over-long escape prefix
(malformed: VC_ERR_FORMAT)."""
import hashlib
import struct

import numpy as np
import pytest

from conftest import load_archive
from test_gpu_decode import STORED, _slot_offset
from rcstream import hostile_payload

pytestmark = pytest.mark.gpu


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


@pytest.fixture
def lockstep(vc, gpu):
    vc.lib().vcg_set_rc_scalar_warps(0)
    yield
    vc.lib().vcg_set_rc_scalar_warps(-1)


@pytest.mark.parametrize("name", STORED)
def test_lockstep_decoder_matches_reference(vc, golden, lockstep, name):
    c = golden[name]
    a = vc.Archive(load_archive(c))
    for lod, h in enumerate(c["lod_sha256"]):
        s, vol = a.decode_lod(lod)
        assert s == 0 and sha(vol) == h, lod
    for r in c["regions"]:
        s, out = a.decode_region(r["lod"], tuple(r["box"]))
        assert s == r["status"] and sha(out) == r["sha256"]


def test_lockstep_decoder_corrupt_payloads_match_oracle(vc, oracle, golden, lockstep):
    base = bytearray(load_archive(golden["synth_prime_97x131x65_t20"]))
    rng = np.random.default_rng(2024)
    atoms = [(0, 0, 0), (1, 2, 1), (0, 3, 2), (1, 0, 3)]
    for trial in range(8):
        data = bytearray(base)
        for (az, ay, ax) in atoms:
            so = _slot_offset(data, 0, az, ay, ax)
            off, ln = struct.unpack_from("<QI", data, so)
            k = int(rng.integers(1, ln))
            if trial % 2:
                data[off + k: off + ln] = bytes([int(rng.integers(0, 256))]) * (ln - k)
            else:
                data[off + k: off + ln] = rng.integers(0, 256, ln - k).astype(np.uint8).tobytes()
        data = bytes(data)
        a, o = vc.Archive(data), oracle.Archive(data)
        for lod in range(o.nlod):
            s1, g = a.decode_lod(lod)
            s2, r = o.decode_lod(lod)
            assert s1 == s2, (trial, lod)
            if s1 == 0:
                assert (g == r).all(), (trial, lod)


def test_lockstep_decoder_rejects_overlong_escape(vc, oracle, golden, lockstep):
    """An atom whose payload is replaced (in place, same length budget) by a
    stream with a 40-one escape prefix: the oracle and the GPU report
    VC_ERR_FORMAT for the LOD and for that atom, and decode the atoms before it
    in (z, y, x) order identically."""
    data = bytearray(load_archive(golden["synth_prime_97x131x65_t20"]))
    bad = hostile_payload()
    so = _slot_offset(data, 0, 1, 2, 1)
    off, ln = struct.unpack_from("<QI", data, so)
    assert ln >= len(bad)
    data[off:off + len(bad)] = bad
    struct.pack_into("<I", data, so + 8, len(bad))
    data = bytes(data)
    a, o = vc.Archive(data), oracle.Archive(data)
    box = (0, 0, 0, 97, 131, 65)
    g = np.full(97 * 131 * 65, 0x5A, np.uint8)
    r = g.copy()
    s1, _ = a.decode_region(0, box, g)
    s2, _ = o.decode_region(0, box, r)
    assert s1 == s2 == vc.VC_ERR_FORMAT
    assert (g == r).all()
    s1, at = a.decode_atom(0, 1, 2, 1)
    s2, at2 = o.decode_atom(0, 1, 2, 1)
    assert s1 == s2 == vc.VC_ERR_FORMAT and (at == 0).all() and (at2 == 0).all()


def test_lockstep_decoder_truncated_archive_matches_oracle(vc, oracle, golden, lockstep):
    data = load_archive(golden["synth_prime_97x131x65_t20"])
    for cut in [len(data) - 1, len(data) - 3000, 650000]:
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
