"""vcg_decode_atoms_noalloc — the decode entry point that allocates nothing,
for callers that cannot let a library allocate device memory (applications
that reserve the whole GPU for their own pool, or that cannot afford the
synchronisation cudaMalloc / cudaFree may cause). Its output must equal the
regular vc_decode_atom output exactly, on two calls in a row (the calls share
one fixed scratch array, so the second must not see the first's leftovers).

This file is named to be collected last."""
import struct

import numpy as np
import pytest

from conftest import load_archive

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
