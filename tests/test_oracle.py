"""Pins the CPU oracle: against the golden fixtures produced by the reference
codec (everywhere) and against the reference build itself (where it exists)."""
import hashlib

import numpy as np
import pytest

from conftest import load_archive

SYNTH = ["synth_64_t10", "synth_prime_97x131x65_t20", "synth_flat_96x64x33_t100", "synth_thin_2048x32x32_t50",
         "cfg1_256_t10"]


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


@pytest.fixture(scope="module")
def ref():
    import refcodec
    if not refcodec.available():
        pytest.skip("reference build (oracle/_ref) not present on this host")
    return refcodec


def synth_volume(vc, case):
    nx, ny, nz = case["dims"]
    return vc.synth(nx, ny, nz, case["seed"])


@pytest.mark.parametrize("name", SYNTH)
def test_synth_volume_is_pinned(vc, golden, name):
    assert sha(synth_volume(vc, golden[name])) == golden[name]["volume_sha256"]


@pytest.mark.parametrize("name", SYNTH)
def test_oracle_encode_matches_reference_archive(vc, oracle, golden, name):
    c = golden[name]
    vol = synth_volume(vc, c)
    q0, npres, nbytes = oracle.rate_control(vol, c["target"])
    assert q0 == pytest.approx(c["q0"], rel=0, abs=0)
    s, data = oracle.encode(vol, c["target"])
    assert s == 0 and len(data) == c["len"] and sha(data) == c["sha256"]


@pytest.mark.parametrize("name", ["synth_64_t10", "synth_prime_97x131x65_t20", "tiny_1x1x1",
                                  "synth_flat_96x64x33_t100"])
def test_oracle_decode_matches_reference(oracle, golden, name):
    c = golden[name]
    data = load_archive(c)
    assert sha(data) == c["sha256"]
    a = oracle.Archive(data)
    for lod in range(a.nlod):
        s, vol = a.decode_lod(lod)
        assert s == 0 and sha(vol) == c["lod_sha256"][lod]
        _, (nx, ny, nz) = a.lod_dims(lod)
        h = hashlib.sha256()
        for az in range((nz + 31) // 32):
            for ay in range((ny + 31) // 32):
                for ax in range((nx + 31) // 32):
                    s, at = a.decode_atom(lod, ax, ay, az)
                    assert s == 0
                    h.update(at.tobytes())
        assert h.hexdigest() == c["atoms_sha256"][lod]
    for r in c["regions"]:
        s, out = a.decode_region(r["lod"], tuple(r["box"]))
        assert s == r["status"] and sha(out) == r["sha256"]


@pytest.mark.parametrize("name", ["ref_test_basic", "extreme_zero", "extreme_voxel", "extreme_line", "extreme_sat"])
def test_oracle_reads_reference_writer_archives(oracle, golden, name):
    c = golden[name]
    a = oracle.Archive(load_archive(c))
    nx, ny, nz = c["dims"]
    i = 0
    for az in range((nz + 31) // 32):
        for ay in range((ny + 31) // 32):
            for ax in range((nx + 31) // 32):
                s, at = a.decode_atom(0, ax, ay, az)
                assert s == 0 and sha(at) == c["atom_sha256"][i]
                assert a.coverage(0, az, ay, ax) == c["coverage"][i]
                i += 1
    s, full = a.decode_lod(0)
    assert s == 0 and sha(full) == c["lod0_sha256"]


def test_oracle_fixed_q_archives(vc, oracle, golden):
    c = golden["fixed_q_128"]
    vol = synth_volume(vc, c)
    for run in c["runs"]:
        s, data = oracle.encode_fixed_q(vol, 10.0, [run["q"]] * 8)
        assert s == 0 and sha(data) == run["sha256"], run["q"]


def test_oracle_size_only_coder_matches_writer(oracle):
    rng = np.random.default_rng(3)
    L = oracle.lib()
    for _ in range(20):
        lv = np.zeros(32768, np.int16)
        idx = rng.choice(32768, rng.integers(0, 6000), replace=False)
        lv[idx] = rng.integers(-300, 300, len(idx))
        buf = np.zeros(200000, np.uint8)
        n = L.orc_enc_levels(oracle.ptr(lv), oracle.ptr(buf), len(buf))
        assert L.orc_rc_size(oracle.ptr(lv)) == n
        back = np.zeros(32768, np.int16)
        assert L.orc_dec_levels(oracle.ptr(buf), n, oracle.ptr(back)) == 0
        assert (back == lv).all()


def _atom_kinds(rng):
    z = np.arange(32)[:, None, None]
    y = np.arange(32)[None, :, None]
    x = np.arange(32)[None, None, :]
    s = 16 + 4 * np.sin(2 * np.pi * x / rng.uniform(20, 90)) + 3 * np.sin(2 * np.pi * y / rng.uniform(20, 90))
    sheet = 18 + rng.normal(0, 5, (32, 32, 32)) + np.where(np.abs(z - s) < 3, rng.uniform(110, 170), 0)
    yield np.clip(np.rint(sheet), 0, 255).astype(np.uint8).ravel()
    yield rng.integers(0, 256, 32768).astype(np.uint8)
    v = np.zeros(32768, np.uint8)
    v[rng.integers(0, 32768, 3)] = 250
    yield v
    yield np.full(32768, 255, np.uint8)


def test_oracle_kernels_match_reference(oracle, ref):
    import ctypes
    R = ref.lib()
    O = oracle.lib()
    R.refshim_encode_atom.restype = ctypes.c_uint32
    rng = np.random.default_rng(11)
    p = oracle.ptr
    for it in range(12):
        q = np.float32(np.exp(rng.uniform(np.log(0.05), np.log(4096))))
        for vox in _atom_kinds(rng):
            dc = int((int(vox.astype(np.uint32).sum()) + 16384) // 32768)
            c1, c2 = np.zeros(32768, np.int32), np.zeros(32768, np.int32)
            R.refshim_fdct(p(vox), dc, p(c1))
            O.orc_fdct(p(vox), dc, p(c2))
            assert (c1 == c2).all()
            l1, l2 = np.zeros(32768, np.int16), np.zeros(32768, np.int16)
            R.refshim_quantize(p(c1), ctypes.c_float(q), p(l1))
            O.orc_quantize(p(c1), ctypes.c_float(q), p(l2))
            assert (l1 == l2).all()
            d1, d2 = np.zeros(32768, np.int32), np.zeros(32768, np.int32)
            R.refshim_dequantize(p(l1), ctypes.c_float(q), p(d1))
            O.orc_dequantize(p(l1), ctypes.c_float(q), p(d2))
            assert (d1 == d2).all()
            v1, v2 = np.zeros(32768, np.uint8), np.zeros(32768, np.uint8)
            R.refshim_idct(p(d1), dc, p(v1))
            O.orc_idct(p(d1), dc, p(v2))
            assert (v1 == v2).all()
            b1, b2 = np.zeros(140000, np.uint8), np.zeros(140000, np.uint8)
            z1, z2, e1, e2 = ctypes.c_int(), ctypes.c_int(), ctypes.c_uint8(), ctypes.c_uint8()
            n1 = R.refshim_encode_atom(p(vox), ctypes.c_float(q), p(b1), len(b1), ctypes.byref(z1), ctypes.byref(e1))
            n2 = O.orc_encode_atom(p(vox), ctypes.c_float(q), p(b2), len(b2), ctypes.byref(z2), ctypes.byref(e2))
            assert n1 == n2 and (b1[:n1] == b2[:n2]).all()


def test_oracle_tables_match_reference(oracle, ref):
    import ctypes
    R = ref.lib()
    cm1, cm2 = np.zeros(1024, np.int32), np.zeros(1024, np.int32)
    st1, st2 = np.zeros(32768, np.float32), np.zeros(32768, np.float32)
    sc1, sc2 = np.zeros(32768, np.uint16), np.zeros(32768, np.uint16)
    R.refshim_tables(oracle.ptr(cm1), oracle.ptr(st1), oracle.ptr(sc1))
    oracle.lib().orc_tables(oracle.ptr(cm2), oracle.ptr(st2), oracle.ptr(sc2))
    assert (cm1 == cm2).all() and (st1.view(np.uint32) == st2.view(np.uint32)).all() and (sc1 == sc2).all()
    for q in [0.05, 0.7, 1.0, 3.3, 100.0, 4096.0]:
        a1, b1 = np.zeros(32768, np.int32), np.zeros(32768, np.int32)
        a2, b2 = np.zeros(32768, np.int32), np.zeros(32768, np.int32)
        R.refshim_dq_tables(ctypes.c_float(q), oracle.ptr(a1), oracle.ptr(b1))
        oracle.lib().orc_dq_tables(ctypes.c_float(q), oracle.ptr(a2), oracle.ptr(b2))
        assert (a1 == a2).all() and (b1 == b2).all()


def test_oracle_encode_random_dims_matches_reference(oracle, ref):
    rng = np.random.default_rng(21)
    for _ in range(6):
        nx, ny, nz = (int(v) for v in rng.integers(1, 80, 3))
        vol = np.clip(rng.normal(90, 40, (nz, ny, nx)), 0, 255).astype(np.uint8)
        vol[vol < 60] = 0
        t = float(rng.choice([10.0, 20.0, 50.0]))
        data_ref, q0 = ref.ref_encode(vol, t)
        s, data = oracle.encode(vol, t)
        assert s == 0 and data == data_ref, (nx, ny, nz, t)


def test_forward_coefficients_fit_seventeen_bits(oracle):
    """The GPU rate-control quantiser keeps each LOD0 coefficient packed with
    its class and sign, the magnitude in 17 bits. The transform of 8-bit voxels
    minus any centre in [0, 255] stays far below 2^17: the largest magnitude is
    the DC coefficient of a block at 255 above or below its centre, 46,132 (the
    DC row of the matrix has the largest absolute sum, 32 x 2896), and no
    extreme pattern exceeds it."""
    import ctypes
    L = oracle.lib()
    rng = np.random.default_rng(17)
    x, y, z = np.meshgrid(np.arange(32), np.arange(32), np.arange(32), indexing="xy")
    patterns = [np.full(32768, 255, np.uint8), np.zeros(32768, np.uint8),
                (((x + y + z) & 1) * 255).astype(np.uint8).ravel(), ((x & 1) * 255).astype(np.uint8).ravel(),
                ((((x >> 2) + (y >> 3) + z) & 1) * 255).astype(np.uint8).ravel()]
    patterns += [(rng.integers(0, 2, 32768) * 255).astype(np.uint8) for _ in range(6)]
    one = np.zeros(32768, np.uint8)
    one[0] = 255
    patterns.append(one)
    peak = 0
    coef = np.zeros(32768, np.int32)
    for vox in patterns:
        for dc in (0, 128, 255):
            L.orc_fdct(vox.ctypes.data, ctypes.c_int32(dc), coef.ctypes.data)
            peak = max(peak, int(np.abs(coef).max()))
    dc_peak = 0
    for v, c in ((255, 0), (0, 255)):   # 255 above and below the centre
        block = np.full(32768, v, np.uint8)
        L.orc_fdct(block.ctypes.data, ctypes.c_int32(c), coef.ctypes.data)
        dc_peak = max(dc_peak, int(abs(coef[0])))
    assert dc_peak == 46132
    assert peak == dc_peak
    assert peak < (1 << 17)
