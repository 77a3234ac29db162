"""Solo atoms (vcg_set_rc_solo): the per-lane range decoder's longest atoms on
latency-decoder warps of their own, on a second stream beside it. LOD0 of the
1024^3 archive at target 10 (32,768 atoms: the per-lane decoder) decoded with
76 solo atoms and with every atom solo (no per-lane launch at all), into host
and device memory, must give the reference's bytes."""
import hashlib

import pytest

pytestmark = pytest.mark.gpu


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


def test_solo_atoms_decode_like_reference(vc, gpu, golden):
    name = "cfg2_1024_t10"
    if name not in golden:
        pytest.skip("1024^3 golden archive not generated")
    c = golden[name]
    nx, ny, nz = c["dims"]
    dbuf = vc.synth_device(nx, ny, nz, c["seed"])
    s, data, _ = vc.encode_device(dbuf, (nx, ny, nz), c["target"])
    assert s == 0 and sha(data) == c["sha256"]
    a = vc.Archive(data)
    for n in (76, 1 << 30):
        vc.lib().vcg_set_rc_solo(n)
        try:
            s, v = a.decode_lod(0)
            assert s == 0 and sha(v) == c["lod_sha256"][0], n
            assert a.decode_lod_device(0, dbuf) == 0
            assert sha(dbuf.download(nx * ny * nz)) == c["lod_sha256"][0], n
        finally:
            vc.lib().vcg_set_rc_solo(-1)
    dbuf.free()
