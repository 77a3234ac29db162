"""The batched / served workload at its full size, pinned to the reference: the
2048x2048x1536 synthetic volume encoded at target_ratio 20 must give the
reference's archive, and the first boxes of the workload's box list (LOD
U{0..3}, edges U[32,256]) decoded in one batch, through the serving loop and
one at a time must give the reference's bytes (golden hashes generated by
tests/golden/gen_golden.py --cfg4 from the reference's own decoder)."""
import hashlib

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

NAME = "cfg4_2048x2048x1536_t20"


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


def box_bytes(b):
    return (b[3] - b[0]) * (b[4] - b[1]) * (b[5] - b[2])


@pytest.fixture(scope="module")
def cfg4(vc, gpu, golden):
    if NAME not in golden:
        pytest.skip("2048x2048x1536 golden case not generated")
    c = golden[NAME]
    nx, ny, nz = c["dims"]
    dv = vc.synth_device(nx, ny, nz, c["seed"])
    s, data, q0 = vc.encode_device(dv, (nx, ny, nz), c["target"])
    dv.free()
    assert s == 0, vc.last_error()
    return c, data, q0


def test_cfg4_archive_is_the_references(cfg4):
    c, data, q0 = cfg4
    assert q0 == c["q0"] and len(data) == c["len"] and sha(data) == c["sha256"]


def test_cfg4_batched_boxes_match_reference(vc, cfg4):
    c, data, _ = cfg4
    a = vc.Archive(data)
    reqs = [(b["lod"], tuple(b["box"])) for b in c["boxes"]]
    outs = [vc.DeviceBuffer(box_bytes(b)) for _, b in reqs]
    s, st = a.decode_regions(reqs, outs, True)
    assert s == vc.VC_OK and (np.asarray(st) == 0).all()
    for i, b in enumerate(c["boxes"]):
        assert sha(outs[i].download(box_bytes(b["box"]))) == b["sha256"], i
    for o in outs:
        o.free()
    # host outputs, second batch (graph replay)
    outs = [np.zeros(box_bytes(b), np.uint8) for _, b in reqs]
    s, st = a.decode_regions(reqs, outs, False)
    assert s == vc.VC_OK
    for i, b in enumerate(c["boxes"]):
        assert sha(outs[i]) == b["sha256"], i


def test_cfg4_served_boxes_match_reference(vc, cfg4):
    c, data, _ = cfg4
    a = vc.Archive(data)
    outs = [np.zeros(box_bytes(b["box"]), np.uint8) for b in c["boxes"]]
    with a.server(device_budget=2 << 30, max_batch=256, workers=2) as srv:
        tix = [srv.submit(b["lod"], tuple(b["box"]), o) for b, o in zip(c["boxes"], outs)]
        res = [srv.wait(t) for t in tix]
    assert all(r[0] == vc.VC_OK for r in res)
    for i, b in enumerate(c["boxes"]):
        assert sha(outs[i]) == b["sha256"], i


def test_cfg4_plain_boxes_match_reference(vc, cfg4):
    c, data, _ = cfg4
    a = vc.Archive(data)
    for b in c["boxes"][:40]:
        s, out = a.decode_region(b["lod"], tuple(b["box"]))
        assert s == vc.VC_OK and sha(out) == b["sha256"]
