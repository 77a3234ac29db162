"""The served workload at its full size, pinned to the reference: the 2048^3
synthetic volume encoded at target_ratio 20 must give the reference's archive,
and the first requests of the served mix (70 % single 32^3 atoms at LOD0, 25 %
boxes with edges U[64,128] at LOD 0-1, 5 % 512^3 boxes at LOD2) decoded through
the serving loop, in one batch and one at a time must give the reference's
bytes (golden hashes generated by tests/golden/gen_golden.py --cfg5 from the
reference's own decoder)."""
import hashlib

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

NAME = "cfg5_2048_t20"


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


def box_bytes(b):
    return (b[3] - b[0]) * (b[4] - b[1]) * (b[5] - b[2])


@pytest.fixture(scope="module")
def cfg5(vc, gpu, golden):
    if NAME not in golden:
        pytest.skip("2048^3 golden case not generated")
    c = golden[NAME]
    nx, ny, nz = c["dims"]
    dv = vc.synth_device(nx, ny, nz, c["seed"])
    s, data, q0 = vc.encode_device(dv, (nx, ny, nz), c["target"])
    dv.free()
    assert s == 0, vc.last_error()
    return c, data, q0


def test_cfg5_archive_is_the_references(cfg5):
    c, data, q0 = cfg5
    assert q0 == c["q0"] and len(data) == c["len"] and sha(data) == c["sha256"]


def test_cfg5_served_requests_match_reference(vc, cfg5):
    c, data, _ = cfg5
    a = vc.Archive(data)
    reqs = c["requests"]
    outs = [np.zeros(box_bytes(r["box"]), np.uint8) for r in reqs]
    with a.server(device_budget=2 << 30, max_batch=1024, workers=3) as srv:
        tix = [srv.submit(r["lod"], tuple(r["box"]), o) for r, o in zip(reqs, outs)]
        res = [srv.wait(t) for t in tix]
    assert all(r[0] == vc.VC_OK for r in res)
    for i, r in enumerate(reqs):
        assert sha(outs[i]) == r["sha256"], i


def test_cfg5_batched_and_plain_requests_match_reference(vc, cfg5):
    c, data, _ = cfg5
    a = vc.Archive(data)
    reqs = c["requests"]
    outs = [np.zeros(box_bytes(r["box"]), np.uint8) for r in reqs]
    s, st = a.decode_regions([(r["lod"], tuple(r["box"])) for r in reqs], outs, False)
    assert s == vc.VC_OK and (np.asarray(st) == 0).all()
    for i, r in enumerate(reqs):
        assert sha(outs[i]) == r["sha256"], i
    for r in reqs[:40]:
        s, out = a.decode_region(r["lod"], tuple(r["box"]))
        assert s == vc.VC_OK and sha(out) == r["sha256"]
