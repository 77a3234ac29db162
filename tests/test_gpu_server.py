"""Decode server (vcg_server_*): requests submitted from several host threads
into the continuous-batching loop come back with exactly the status and bytes
the oracle's vc_decode_region gives for that request alone, under a
device-memory budget that forces admission to wait, with batches of several
workers in flight."""
import struct
import threading

import numpy as np
import pytest

from conftest import load_archive
from test_gpu_batch import box_bytes, oracle_of, random_requests


def run_mixed(vc, a, reqs, threads, budget, max_batch, workers):
    outs = [np.full(max(1, box_bytes(b)), 0x5A, np.uint8) for _, b in reqs]
    res = [None] * len(reqs)
    with a.server(device_budget=budget, max_batch=max_batch, workers=workers) as srv:
        def client(k):
            mine = list(range(k, len(reqs), threads))
            tix = [srv.submit(reqs[i][0], reqs[i][1], outs[i]) for i in mine]
            for i, t in zip(mine, tix):
                assert t >= 0
                res[i] = srv.wait(t)
        th = [threading.Thread(target=client, args=(k,)) for k in range(threads)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        batches, done = srv.stats()
    assert done == len(reqs)
    return outs, res, batches


def check_alone(vc, a, reqs, outs, res):
    o = oracle_of(a)
    for i, (lod, box) in enumerate(reqs):
        ref = np.full(max(1, box_bytes(box)), 0x5A, np.uint8)
        s, _ = o.decode_region(lod, box, ref)
        assert res[i][0] == s, (i, lod, box)
        assert res[i][1] >= 0.0
        if s == vc.VC_OK:
            assert np.array_equal(outs[i], ref), (i, lod, box)


@pytest.mark.gpu
@pytest.mark.parametrize("budget,max_batch,workers", [(1 << 30, 4096, 2), (600_000, 64, 3), (1, 8, 1)])
def test_server_mix_equals_alone(vc, gpu, golden, budget, max_batch, workers):
    data = load_archive(golden["synth_prime_97x131x65_t20"])
    a = vc.Archive(data)
    nlod = struct.unpack_from("<I", data, 20)[0]
    reqs = random_requests(a, np.random.default_rng(21), 240, min(nlod - 1, 3), max_edge=97, invalid=4)
    outs, res, batches = run_mixed(vc, a, reqs, threads=4, budget=budget, max_batch=max_batch, workers=workers)
    check_alone(vc, a, reqs, outs, res)
    assert batches >= -(-len(reqs) // max_batch)
    if budget == 1:
        # every non-empty box exceeds the budget and runs alone; empty boxes hold
        # no device memory, so two of them that meet in the queue may share a batch
        n_boxes = sum(1 for _, b in reqs if box_bytes(b) > 0)
        assert n_boxes <= batches <= len(reqs)


@pytest.mark.gpu
def test_server_on_corrupt_archive(vc, gpu, golden):
    from test_gpu_decode import _slot_offset
    data = bytearray(load_archive(golden["synth_prime_97x131x65_t20"]))
    so = _slot_offset(data, 0, 1, 2, 1)
    struct.pack_into("<I", data, so + 8, len(data))
    a = vc.Archive(bytes(data))
    reqs = random_requests(a, np.random.default_rng(22), 80, 1, max_edge=97) + [(0, (0, 0, 0, 97, 131, 65))]
    outs, res, _ = run_mixed(vc, a, reqs, threads=3, budget=4 << 20, max_batch=16, workers=2)
    check_alone(vc, a, reqs, outs, res)
    assert any(r[0] == vc.VC_ERR_FORMAT for r in res)


@pytest.mark.gpu
def test_server_destroy_drains_queue(vc, gpu, golden):
    a = vc.Archive(load_archive(golden["synth_64_t10"]))
    reqs = random_requests(a, np.random.default_rng(23), 50, 1, max_edge=64)
    outs = [np.zeros(max(1, box_bytes(b)), np.uint8) for _, b in reqs]
    srv = a.server(device_budget=1 << 20, max_batch=4, workers=2)
    for (lod, box), o in zip(reqs, outs):
        assert srv.submit(lod, box, o) >= 0
    srv.close()   # returns only after every queued request ran
    ora = oracle_of(a)
    for (lod, box), o in zip(reqs, outs):
        ref = np.zeros(max(1, box_bytes(box)), np.uint8)
        s, _ = ora.decode_region(lod, box, ref)
        assert s == vc.VC_OK and np.array_equal(o, ref)


def test_server_host_logic_without_device(vc, golden):
    """Queue, admission and wait bookkeeping; without a GPU each request carries
    the decode call's VC_ERR_IO, with a GPU its plain status."""
    a = vc.Archive(load_archive(golden["synth_64_t10"]))
    reqs = random_requests(a, np.random.default_rng(24), 30, 1, max_edge=64, invalid=2)
    outs, res, batches = run_mixed(vc, a, reqs, threads=3, budget=1 << 16, max_batch=5, workers=2)
    assert batches >= 6
    statuses = {r[0] for r in res}
    assert statuses <= {vc.VC_OK, vc.VC_ERR_RANGE, vc.VC_ERR_IO}
    with pytest.raises(RuntimeError):
        a.server(device_budget=0)
    with a.server() as srv:
        assert srv.wait(5)[0] == vc.VC_ERR_RANGE   # ticket never issued
    # slots of waited tickets are recycled: thousands of tickets, a second wait is refused
    out = np.zeros(32768, np.uint8)
    with a.server(device_budget=1 << 20, max_batch=16, workers=2) as srv:
        first = srv.submit(0, (0, 0, 0, 32, 32, 32), out)
        assert srv.wait(first)[0] in (vc.VC_OK, vc.VC_ERR_IO)
        assert srv.wait(first)[0] == vc.VC_ERR_RANGE
        for _ in range(30):
            tix = [srv.submit(0, (0, 0, 0, 32, 32, 32), out) for _ in range(100)]
            assert all(t >= 0 for t in tix)
            assert {srv.wait(t)[0] for t in tix} <= {vc.VC_OK, vc.VC_ERR_IO}
        assert srv.wait(first)[0] == vc.VC_ERR_RANGE
        batches, done = srv.stats()
        assert done == 3001
