"""GPU encode parity: vc_encode produces byte-identical archives to the
reference composition (golden hashes) and to the oracle, at explicit q values
across the whole clamp range, and for edge-case volumes."""
import hashlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SYNTH = ["synth_64_t10", "synth_prime_97x131x65_t20", "synth_flat_96x64x33_t100", "synth_thin_2048x32x32_t50",
         "cfg1_256_t10"]


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


@pytest.mark.parametrize("name", SYNTH)
def test_encode_is_byte_identical_to_reference(vc, gpu, golden, name):
    c = golden[name]
    nx, ny, nz = c["dims"]
    vol = vc.synth(nx, ny, nz, c["seed"])
    s, data = vc.encode(vol, c["target"])
    assert s == 0 and len(data) == c["len"] and sha(data) == c["sha256"]
    a = vc.Archive(data)
    for lod, h in enumerate(c["lod_sha256"]):
        s, v = a.decode_lod(lod)
        assert s == 0 and sha(v) == h, lod


def test_device_input_and_device_synth(vc, gpu, golden):
    c = golden["cfg1_256_t10"]
    nx, ny, nz = c["dims"]
    dbuf = vc.synth_device(nx, ny, nz, c["seed"])
    assert sha(dbuf.download(nx * ny * nz)) == c["volume_sha256"]
    s, data, q0 = vc.encode_device(dbuf, (nx, ny, nz), c["target"])
    assert s == 0 and sha(data) == c["sha256"] and q0 == c["q0"]


def test_fixed_q_archives(vc, gpu, golden):
    c = golden["fixed_q_128"]
    nx, ny, nz = c["dims"]
    vol = vc.synth(nx, ny, nz, c["seed"])
    for run in c["runs"]:
        s, data = vc.encode_q(vol, 10.0, [run["q"]] * 8)
        assert s == 0 and sha(data) == run["sha256"], run["q"]


def test_random_volumes_match_oracle(vc, oracle, gpu):
    rng = np.random.default_rng(5)
    for _ in range(8):
        nx, ny, nz = (int(v) for v in rng.integers(1, 150, 3))
        vol = np.clip(rng.normal(100, 50, (nz, ny, nx)), 0, 255).astype(np.uint8)
        vol[vol < 70] = 0
        t = float(rng.choice([1.0, 10.0, 33.0, 100.0]))
        s1, g = vc.encode(vol, t)
        s2, r = oracle.encode(vol, t)
        assert s1 == s2 == 0 and g == r, (nx, ny, nz, t)


@pytest.mark.parametrize("kind", ["zero", "sat", "voxel", "noise"])
def test_edge_volumes_match_oracle(vc, oracle, gpu, kind):
    vol = np.zeros((70, 40, 33), np.uint8)
    if kind == "sat":
        vol[:] = 255
    elif kind == "voxel":
        vol[5, 5, 5] = 200
    elif kind == "noise":
        vol = np.random.default_rng(1).integers(0, 256, vol.shape).astype(np.uint8)
    for t in (1.0, 10.0):
        s1, g = vc.encode(vol, t)
        s2, r = oracle.encode(vol, t)
        assert s1 == s2 == 0 and g == r, (kind, t)
    # lowest q: the largest levels the quantiser can produce
    s1, g = vc.encode_q(vol, 1.0, [0.05] * 8)
    s2, r = oracle.encode_fixed_q(vol, 1.0, [0.05] * 8)
    assert s1 == s2 == 0 and g == r


@pytest.mark.parametrize("t", [10, 50, 100])
def test_config2_1024_archives_match_reference(vc, gpu, golden, t):
    name = f"cfg2_1024_t{t}"
    if name not in golden:
        pytest.skip("1024^3 golden archive not generated")
    c = golden[name]
    nx, ny, nz = c["dims"]
    dbuf = vc.synth_device(nx, ny, nz, c["seed"])
    s, data, q0 = vc.encode_device(dbuf, (nx, ny, nz), c["target"])
    assert s == 0 and q0 == c["q0"] and len(data) == c["len"] and sha(data) == c["sha256"]
    a = vc.Archive(data)
    for lod, h in enumerate(c["lod_sha256"]):
        s, v = a.decode_lod(lod)
        assert s == 0 and sha(v) == h, lod
    for r in c["regions"]:
        s, out = a.decode_region(r["lod"], tuple(r["box"]))
        assert s == 0 and sha(out) == r["sha256"]
