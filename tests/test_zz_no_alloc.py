"""vcg_decode_atoms_noalloc — the decode entry point that allocates nothing,
for callers that cannot let a library allocate device memory (applications
that reserve the whole GPU for their own pool, or that cannot afford the
synchronisation cudaMalloc / cudaFree may cause). Its output must equal the
regular vc_decode_atom output exactly, on two calls in a row (the calls share
one fixed scratch array, so the second must not see the first's leftovers).

This file is named to be collected last."""
import ctypes
import struct

import numpy as np
import pytest

from conftest import load_archive
from rcstream import hostile_payload

pytestmark = pytest.mark.gpu


def _atoms(a, lod, limit):
    _, (nx, ny, nz) = a.lod_dims(lod)
    out = []
    for az in range((nz + 31) // 32):
        for ay in range((ny + 31) // 32):
            for ax in range((nx + 31) // 32):
                out.append((az, ay, ax))
    return out[:limit]


def test_noalloc_decode_equals_regular_decode_on_two_calls(vc, gpu, golden):
    data = load_archive(golden["synth_prime_97x131x65_t20"])
    a = vc.Archive(data)
    dev = vc.DeviceBuffer(len(data))
    dev.upload(np.frombuffer(data, np.uint8))
    base_q = struct.unpack_from("<8f", data, 72)
    L = vc.lib()
    for lod in (0, 1):   # two calls in a row, different atom sets and q
        atoms = _atoms(a, lod, 64)
        offs = np.zeros(len(atoms), np.uint64)
        lens = np.zeros(len(atoms), np.uint32)
        for i, (az, ay, ax) in enumerate(atoms):
            cov, o, n = a.payload_range(lod, az, ay, ax)
            offs[i], lens[i] = o, n
        out = vc.DeviceBuffer(len(atoms) * 32768)
        s = L.vcg_decode_atoms_noalloc(dev.ptr, len(data), vc.ptr(offs), vc.ptr(lens), len(atoms),
                                       base_q[lod], out.ptr)
        assert s == vc.VC_OK, vc.last_error()
        got = out.download().reshape(len(atoms), 32768)
        for i, (az, ay, ax) in enumerate(atoms):
            s, ref = a.decode_atom(lod, ax, ay, az)
            assert s == vc.VC_OK
            assert np.array_equal(got[i], ref), (lod, az, ay, ax)


def test_noalloc_rejects_more_than_its_limit(vc, gpu):
    L = vc.lib()
    buf = vc.DeviceBuffer(1 << 16)
    offs = np.zeros(65, np.uint64)
    lens = np.ones(65, np.uint32)
    assert L.vcg_decode_atoms_noalloc(buf.ptr, 1 << 16, vc.ptr(offs), vc.ptr(lens), 65, 1.0, buf.ptr) == \
        vc.VC_ERR_RANGE
    offs[0] = (1 << 16) - 1
    lens[0] = 8
    assert L.vcg_decode_atoms_noalloc(buf.ptr, 1 << 16, vc.ptr(offs), vc.ptr(lens), 1, 1.0, buf.ptr) == \
        vc.VC_ERR_FORMAT


def _payloads(a, data, lod, atoms):
    offs = np.zeros(len(atoms), np.uint64)
    lens = np.zeros(len(atoms), np.uint32)
    for i, (az, ay, ax) in enumerate(atoms):
        cov, o, n = a.payload_range(lod, az, ay, ax)
        offs[i], lens[i] = o, n
    return offs, lens


def test_noalloc_rejects_a_malformed_payload_then_decodes_correctly(vc, oracle, gpu, golden):
    """A payload inside the buffer whose coder stream is malformed gives
    VC_ERR_FORMAT (the oracle rejects it too); the scratch it leaves behind must
    not change the next, correct call, which still equals vc_decode_atom."""
    data = load_archive(golden["synth_prime_97x131x65_t20"])
    bad = hostile_payload()
    out = np.zeros(32768, np.uint8)
    assert oracle.lib().orc_decode_atom_payload(bad, len(bad), ctypes.c_float(1.0), vc.ptr(out)) == 1
    a = vc.Archive(data)
    base_q = struct.unpack_from("<8f", data, 72)
    pad = (-len(data)) % 4
    buf = np.frombuffer(data + bytes(pad) + bad, np.uint8)
    dev = vc.DeviceBuffer(len(buf))
    dev.upload(buf)
    L = vc.lib()
    atoms = _atoms(a, 0, 8)
    offs, lens = _payloads(a, data, 0, atoms)
    res = vc.DeviceBuffer(len(atoms) * 32768)
    offs_bad, lens_bad = offs.copy(), lens.copy()
    offs_bad[3], lens_bad[3] = len(data) + pad, len(bad)
    s = L.vcg_decode_atoms_noalloc(dev.ptr, len(buf), vc.ptr(offs_bad), vc.ptr(lens_bad), len(atoms),
                                   base_q[0], res.ptr)
    assert s == vc.VC_ERR_FORMAT
    assert vc.last_error()
    s = L.vcg_decode_atoms_noalloc(dev.ptr, len(buf), vc.ptr(offs), vc.ptr(lens), len(atoms), base_q[0], res.ptr)
    assert s == vc.VC_OK, vc.last_error()
    got = res.download().reshape(len(atoms), 32768)
    for i, (az, ay, ax) in enumerate(atoms):
        s, ref = a.decode_atom(0, ax, ay, az)
        assert s == vc.VC_OK and np.array_equal(got[i], ref), (az, ay, ax)


def test_noalloc_allocates_no_device_memory(vc, gpu, golden):
    """After the first call on the device (which sets up the scratch array),
    repeated calls leave the device's free memory exactly where it was."""
    data = load_archive(golden["synth_prime_97x131x65_t20"])
    a = vc.Archive(data)
    dev = vc.DeviceBuffer(len(data))
    dev.upload(np.frombuffer(data, np.uint8))
    base_q = struct.unpack_from("<8f", data, 72)
    L = vc.lib()
    calls = []
    for lod in (0, 1, 0, 2):
        atoms = _atoms(a, lod, 64)
        offs, lens = _payloads(a, data, lod, atoms)
        calls.append((lod, offs, lens, len(atoms)))
    out = vc.DeviceBuffer(64 * 32768)
    lod, offs, lens, n = calls[0]
    assert L.vcg_decode_atoms_noalloc(dev.ptr, len(data), vc.ptr(offs), vc.ptr(lens), n, base_q[lod], out.ptr) == 0
    assert vc.sync() == 0
    s, free0, _ = vc.device_memory()
    assert s == 0
    for _ in range(3):
        for lod, offs, lens, n in calls:
            s = L.vcg_decode_atoms_noalloc(dev.ptr, len(data), vc.ptr(offs), vc.ptr(lens), n, base_q[lod], out.ptr)
            assert s == vc.VC_OK, vc.last_error()
    assert vc.sync() == 0
    s, free1, _ = vc.device_memory()
    assert s == 0
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
