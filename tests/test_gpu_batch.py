"""Batched region decode (vcg_decode_regions): every request equals what the
oracle's vc_decode_region gives for it alone (status and bytes, including the
partial output of a request stopped by a malformed atom), for host and device
outputs, across graph replays, buffer growth, every launch shape and a corrupt
archive."""
import struct

import numpy as np
import pytest

from conftest import load_archive

pytestmark = pytest.mark.gpu


def random_requests(a, rng, n, max_lod, max_edge=90, invalid=0):
    reqs = []
    for _ in range(n):
        lod = int(rng.integers(0, max_lod + 1))
        _, d = a.lod_dims(lod)
        e = [int(rng.integers(1, min(max_edge, d[k]) + 1)) for k in range(3)]
        o = [int(rng.integers(0, d[k] - e[k] + 1)) for k in range(3)]
        reqs.append((lod, (o[0], o[1], o[2], o[0] + e[0], o[1] + e[1], o[2] + e[2])))
    for _ in range(invalid):
        reqs.insert(int(rng.integers(0, len(reqs) + 1)), (0, (5, 5, 5, 5, 9, 9)))   # empty box -> RANGE
    return reqs


def box_bytes(box):
    x0, y0, z0, x1, y1, z1 = box
    return max(0, (x1 - x0) * (y1 - y0) * (z1 - z0))


def oracle_of(a):
    """The oracle's handle on the same archive bytes as the product's handle a."""
    import oraclelib
    if getattr(a, "_oracle", None) is None:
        a._oracle = oraclelib.Archive(bytes(a.buf.raw))
    return a._oracle


def check(vc, a, reqs, on_device):
    o = oracle_of(a)
    if on_device:
        outs = [vc.DeviceBuffer(max(1, box_bytes(b))) for _, b in reqs]
    else:
        outs = [np.full(max(1, box_bytes(b)), 0x5A, np.uint8) for _, b in reqs]
    s, st = a.decode_regions(reqs, outs, on_device)
    assert s == vc.VC_OK
    for i, (lod, box) in enumerate(reqs):
        ref = np.full(max(1, box_bytes(box)), 0x5A, np.uint8)
        s2, _ = o.decode_region(lod, box, ref)
        assert st[i] == s2, (i, lod, box)
        got = outs[i].download(max(1, box_bytes(box))) if on_device else outs[i]
        if s2 == vc.VC_OK:
            assert np.array_equal(got, ref), (i, lod, box)


@pytest.mark.parametrize("name", ["synth_prime_97x131x65_t20", "ref_test_basic", "synth_64_t10"])
def test_batch_matches_oracle_host_and_device(vc, gpu, golden, name):
    a = vc.Archive(load_archive(golden[name]))
    rng = np.random.default_rng(11)
    nlod = struct.unpack_from("<I", load_archive(golden[name]), 20)[0]
    check(vc, a, random_requests(a, rng, 60, min(nlod - 1, 3), invalid=3), on_device=False)
    check(vc, a, random_requests(a, rng, 60, min(nlod - 1, 3), invalid=2), on_device=True)
    rc, tx, imma = vc.batch_shape()
    assert rc in (1, 4, 16) and tx in (256, 512) and imma in (0, 1)


def test_batch_graph_replay_and_growth(vc, gpu, golden):
    a = vc.Archive(load_archive(golden["synth_prime_97x131x65_t20"]))
    rng = np.random.default_rng(12)
    for n, edge in [(10, 40), (10, 40), (200, 97), (5, 20), (300, 130)]:   # replays, then larger buffers
        check(vc, a, random_requests(a, rng, n, 2, max_edge=edge), on_device=True)


def test_batch_on_corrupt_archive_matches_oracle(vc, gpu, golden):
    from test_gpu_decode import _slot_offset
    data = bytearray(load_archive(golden["synth_prime_97x131x65_t20"]))
    so = _slot_offset(data, 0, 1, 2, 1)   # break the payload range of LOD0 atom (1, 2, 1)
    struct.pack_into("<I", data, so + 8, len(data))
    a = vc.Archive(bytes(data))
    rng = np.random.default_rng(13)
    reqs = random_requests(a, rng, 40, 1, max_edge=97) + [(0, (0, 0, 0, 97, 131, 65))]
    check(vc, a, reqs, on_device=False)
    check(vc, a, reqs, on_device=True)


@pytest.mark.parametrize("shape", [(1, 256, 0), (4, 256, 0), (16, 256, 0), (1, 512, 0), (4, 512, 0), (16, 512, 0),
                                   (1, 256, 1), (4, 256, 1), (16, 256, 1)])
def test_every_launch_shape_matches_oracle(vc, gpu, golden, shape):
    """Each candidate of the autotuner (range-decoder policy x transform size x
    butterfly / int8 tensor-core transform) gives the oracle's bytes and
    statuses, also on a corrupt archive."""
    from test_gpu_decode import _slot_offset
    L = vc.lib()
    assert L.vcg_set_batch_shape(*shape) == 0
    try:
        a = vc.Archive(load_archive(golden["synth_prime_97x131x65_t20"]))
        rng = np.random.default_rng(14)
        check(vc, a, random_requests(a, rng, 40, 2, max_edge=97, invalid=1), on_device=False)
        assert vc.batch_shape() == shape
        data = bytearray(load_archive(golden["synth_prime_97x131x65_t20"]))
        so = _slot_offset(data, 0, 1, 2, 1)
        struct.pack_into("<I", data, so + 8, len(data))
        b = vc.Archive(bytes(data))
        check(vc, b, random_requests(b, rng, 30, 1, max_edge=97) + [(0, (0, 0, 0, 97, 131, 65))], on_device=True)
    finally:
        assert L.vcg_set_batch_shape(0, 0, 0) == 0
    assert L.vcg_set_batch_shape(2, 256, 0) == vc.VC_ERR_RANGE
    assert L.vcg_set_batch_shape(4, 512, 1) == vc.VC_ERR_RANGE


@pytest.mark.parametrize("shape", [(16, 512, 0), (16, 256, 0), (16, 256, 1)])
def test_many_boxes_over_one_atom(vc, gpu, golden, shape):
    """More boxes over one atom than the butterfly transform stages per atom
    (64 windows): the boxes beyond them take the per-row path. Half the windows
    cover all 32 planes of the atom in z, half are cropped in z."""
    L = vc.lib()
    assert L.vcg_set_batch_shape(*shape) == 0
    try:
        a = vc.Archive(load_archive(golden["synth_prime_97x131x65_t20"]))
        rng = np.random.default_rng(15)
        reqs = []
        for i in range(150):   # every box holds voxel (40, 40, 40): LOD0 atom (1, 1, 1) = [32, 64)^3
            x0, y0 = int(rng.integers(0, 41)), int(rng.integers(0, 41))
            x1, y1 = int(rng.integers(41, 98)), int(rng.integers(41, 132))
            if i % 2:
                z0, z1 = int(rng.integers(0, 33)), int(rng.integers(64, 66))
            else:
                z0, z1 = int(rng.integers(33, 41)), int(rng.integers(41, 64))
            reqs.append((0, (x0, y0, z0, x1, y1, z1)))
        check(vc, a, reqs, on_device=True)
        check(vc, a, reqs, on_device=False)
    finally:
        assert L.vcg_set_batch_shape(0, 0, 0) == 0


def test_batch_lane_decoder_matches_oracle(vc, gpu):
    """A batch with more distinct atoms than one per warp (range-decoder policy
    1: above 4 x SMs atoms) goes to the per-lane decoder in payload-length
    order; every request equals the oracle's decode of it alone."""
    n = 512
    dv = vc.synth_device(n, n, n, vc.config_seed(2))
    s, data = vc.encode_q(dv, 20.0, [2.6 * 0.6 ** l for l in range(8)], on_device=(n, n, n))
    assert s == 0
    dv.free()
    a = vc.Archive(data)
    L = vc.lib()
    assert L.vcg_set_batch_shape(1, 512, 0) == 0
    try:
        rng = np.random.default_rng(16)
        reqs = random_requests(a, rng, 400, 0, max_edge=70)
        check(vc, a, reqs, on_device=True)
    finally:
        assert L.vcg_set_batch_shape(0, 0, 0) == 0
