"""The exporter's 2x downscale (tools/downscale.h:29-93): DS_BOX and DS_CBOX.

CPU: the oracle's restatement is pinned to the reference's own downscale
(oracle/_ref/libdsref.so, release flags). This covers random and
deviation-tie cells, cells where a fused and an unfused multiply-add round
apart, and whole volumes through both of the reference's paths: the nz == 2
fast path and the generic path with edge replication. DS_BOX is also checked
to equal the codec's pyramid rule.
GPU: both kernels (vector and any-dims) against the oracle, the cascade
against the reference's fixture hashes, and vcg_encode_ds against archives the
reference writer made from the reference's pyramid (tests/golden/gen_ds.py)."""
import hashlib
import json
import os

import numpy as np
import pytest

import oraclelib as O
from conftest import GOLDEN

DS = {c["name"]: c for c in json.load(open(os.path.join(GOLDEN, "ds.json")))["cases"]}
ALPHAS = [0.5, 0.0, 1.0, 0.3, 0.5943000316619873, 0.123, 2.0, -0.5]
SEPARATING = [0.5943000316619873]


def sha(b):
    return hashlib.sha256(np.ascontiguousarray(b).tobytes()).hexdigest()


def ref():
    import refcodec
    if not os.path.exists(refcodec.DS_SO):
        pytest.skip("reference build not present")
    return refcodec


def cells(rng, n):
    c = rng.integers(0, 256, (n, 8), dtype=np.uint8)
    c[: n // 4] = rng.integers(0, 2, (n // 4, 8), dtype=np.uint8) * rng.integers(1, 256, (n // 4, 1), dtype=np.uint8)
    c[n // 4: n // 2] = (rng.integers(90, 110, (n // 4, 8))).astype(np.uint8)     # near-ties around the mean
    c[n // 2: n // 2 + 8] = 0
    return c


def test_oracle_cell_matches_reference(oracle):
    R = ref()
    rng = np.random.default_rng(7)
    L = O.lib()
    for alpha in ALPHAS:
        for c in cells(rng, 6000):
            for m in (0, 1):
                assert L.orc_ds_cell(c.ctypes.data, m, alpha) == R.ds_cell(c, m, alpha), (list(c), m, alpha)


def separating_cells(alpha):
    """Cells realising (sum, best) pairs at which fma(alpha, best - mean, mean)
    and mean + alpha * (best - mean) round to different bytes: [(cell, fused
    result, unfused result)]."""
    f32 = np.float32
    s = np.arange(1, 2041, dtype=np.float64)[:, None]
    b = np.arange(256, dtype=np.float64)[None, :]
    mean32, d32 = (s * 0.125).astype(f32), (b - s * 0.125).astype(f32)
    vf = (np.float64(f32(alpha)) * d32.astype(np.float64) + mean32.astype(np.float64)).astype(f32)
    vu = (mean32 + (f32(alpha) * d32).astype(f32)).astype(f32)
    fin = lambda v: np.where(v < 0, 0, np.where(v > 255, 255, np.floor((v + f32(0.5)).astype(f32))))
    F, U = fin(vf), fin(vu)
    out = []
    for i, j in np.argwhere(F != U):
        S, B = int(s[i, 0]), int(b[0, j])
        m, k = divmod(S - B, 7)
        if S - B < 0 or m > 255 or (m == 255 and k):
            continue
        c = np.array([B] + [m + 1] * k + [m] * (7 - k), np.uint8)
        if np.abs(8 * c.astype(int) - S).argmax() != 0:
            continue
        out.append((c, int(F[i, j]), int(U[i, j])))
    return out


def separating_volume(alpha, ox, oy, nz):
    """A volume whose every 2x2x2 cell is a separating cell."""
    sep = separating_cells(alpha)
    vol = np.zeros((nz, 2 * oy, 2 * ox), np.uint8)
    for z in range((nz + 1) // 2):
        for y in range(oy):
            for x in range(ox):
                c = sep[(x * 7 + y * 13 + z * 5 + ox) % len(sep)][0]
                for dz in range(min(2, nz - 2 * z)):
                    for dy in (0, 1):
                        for dx in (0, 1):
                            vol[2 * z + dz, 2 * y + dy, 2 * x + dx] = c[dz * 4 + dy * 2 + dx]
    return vol


def test_oracle_cell_matches_reference_where_fma_matters(oracle):
    """The reference's cell function (release flags, -ffp-contract=fast)
    computes the fused form."""
    R = ref()
    L = O.lib()
    sep = separating_cells(SEPARATING[0])
    assert len(sep) > 10
    for c, fused, _ in sep:
        assert L.orc_ds_cell(c.ctypes.data, 1, SEPARATING[0]) == R.ds_cell(c, 1, SEPARATING[0]) == fused


@pytest.mark.parametrize("nz", [2, 3])
def test_oracle_lane_rule_matches_reference(oracle, nz):
    """In the reference's nz == 2 fast path the first 8 * floor(ox / 8) outputs
    of each row are multiplied and added separately, the rest fused; the
    generic path (nz == 3 here) is fused throughout."""
    R = ref()
    a = SEPARATING[0]
    unfused_seen = 0
    for ox in range(1, 41):
        vol = separating_volume(a, ox, 3, nz)
        want = R.ds_downscale2x(vol, 1, a)
        assert np.array_equal(O.ds_downscale2x(vol, 1, a), want), ox
        O.lib().orc_ds_set_fused(0)
        unf = np.zeros((3, ox), np.int64)
        for y in range(3):
            for x in range(ox):
                cell = np.ascontiguousarray(
                    [vol[dz, 2 * y + dy, 2 * x + dx] for dz in (0, 1) for dy in (0, 1) for dx in (0, 1)], np.uint8)
                unf[y, x] = O.lib().orc_ds_cell(cell.ctypes.data, 1, a)   # cell stays alive across the call
        O.lib().orc_ds_set_fused(1)
        unfused_seen += int((want[0] == unf).all(axis=0)[: ox & ~7].sum()) if nz == 2 else 0
    if nz == 2:
        assert unfused_seen > 100


@pytest.mark.parametrize("dims", [(64, 48, 2), (96, 32, 2), (17, 9, 5), (1, 1, 1), (33, 2, 7), (64, 64, 64),
                                  (3, 130, 2), (32, 31, 30)])
def test_oracle_volume_matches_reference(oracle, dims):
    R = ref()
    nx, ny, nz = dims
    rng = np.random.default_rng(nx * 1000 + ny * 10 + nz)
    vol = rng.integers(0, 256, (nz, ny, nx), dtype=np.uint8)
    vol[:, :, : nx // 3] = 0
    for m in (0, 1):
        for a in (0.5, 0.5943000316619873, 1.0):
            assert np.array_equal(O.ds_downscale2x(vol, m, a), R.ds_downscale2x(vol, m, a)), (dims, m, a)


def test_box_is_the_codec_pyramid_rule(oracle):
    rng = np.random.default_rng(3)
    import ctypes
    for _ in range(30):
        nx, ny, nz = (int(v) for v in rng.integers(1, 40, 3))
        vol = rng.integers(0, 256, (nz, ny, nx), dtype=np.uint8)
        codec = np.zeros(((nz + 1) // 2, (ny + 1) // 2, (nx + 1) // 2), np.uint8)
        O.lib().orc_downsample2x(vol.ctypes.data, O.Dims(nx, ny, nz), codec.ctypes.data)
        assert np.array_equal(O.ds_downscale2x(vol, 0, 0.5), codec), (nx, ny, nz)
    del ctypes


def test_fixture_levels_match_oracle(oracle, vc):
    """The fixture's level hashes (reference downscale) are the oracle's cascade."""
    for c in DS.values():
        if c["dims"][0] > 128:
            continue
        lvl = vc.synth(*c["dims"], c["seed"])
        for want in c["level_sha256"]:
            lvl = O.ds_downscale2x(lvl, c["method"], c["alpha"])
            assert sha(lvl) == want, c["name"]


def test_downscale_argument_checks(vc):
    import ctypes
    L = vc.lib()
    buf = np.zeros(8, np.uint8)
    out = np.zeros(1, np.uint8)
    d = vc.Dims(2, 2, 2)
    assert L.vcg_downscale2x(buf.ctypes.data, 0, d, 2, 0.5, out.ctypes.data, None) == vc.VC_ERR_RANGE
    assert L.vcg_downscale2x(buf.ctypes.data, 0, d, 1, float("nan"), out.ctypes.data, None) == vc.VC_ERR_RANGE
    assert L.vcg_downscale2x(buf.ctypes.data, 0, vc.Dims(0, 2, 2), 1, 0.5, out.ctypes.data, None) == vc.VC_ERR_RANGE
    assert L.vcg_downscale2x(None, 0, d, 1, 0.5, out.ctypes.data, None) == vc.VC_ERR_RANGE
    arr = (ctypes.c_void_p * 9)()
    assert L.vcg_downscale_pyramid(buf.ctypes.data, d, 1, 0.5, 9, arr) == vc.VC_ERR_RANGE
    assert L.vcg_downscale_pyramid(buf.ctypes.data, d, 1, 0.5, 1, arr) == vc.VC_ERR_RANGE   # null output


# ----------------------------------------------------------------------------- GPU

@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(64, 48, 2), (256, 130, 67), (96, 33, 5), (17, 9, 5), (1, 1, 1), (33, 2, 7),
                                  (32, 1, 1), (512, 64, 33), (1000, 12, 3), (74, 10, 2), (42, 6, 2),
                                  (64, 7, 2)])
def test_gpu_downscale2x_matches_oracle(vc, gpu, dims):
    nx, ny, nz = dims
    rng = np.random.default_rng(nx + 7 * ny + 11 * nz)
    vol = rng.integers(0, 256, (nz, ny, nx), dtype=np.uint8)
    vol[:, : ny // 2, : nx // 2] = 0
    vol[nz // 2:, :, :] = (rng.integers(0, 2, (nz - nz // 2, ny, nx)) * 200).astype(np.uint8)
    for m in (vc.DS_BOX, vc.DS_CBOX):
        for a in (0.5, 0.5943000316619873, 0.0, 1.0, 2.0):
            s, out = vc.downscale2x(vol, m, a)
            assert s == vc.VC_OK and np.array_equal(out, O.ds_downscale2x(vol, m, a)), (dims, m, a)


@pytest.mark.gpu
@pytest.mark.parametrize("nz", [2, 3])
@pytest.mark.parametrize("ox", [5, 8, 13, 16, 37, 48, 64])
def test_gpu_lane_rule_matches_oracle(vc, gpu, ox, nz):
    a = SEPARATING[0]
    vol = separating_volume(a, ox, 5, nz)
    s, out = vc.downscale2x(vol, vc.DS_CBOX, a)
    assert s == vc.VC_OK and np.array_equal(out, O.ds_downscale2x(vol, 1, a))


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(DS))
def test_gpu_pyramid_and_encode_match_reference(vc, gpu, golden, name):
    c = DS[name]
    nx, ny, nz = c["dims"]
    vol = vc.synth(nx, ny, nz, c["seed"])
    dbuf = vc.DeviceBuffer(nx * ny * nz)
    dbuf.upload(vol)
    levels = len(c["level_sha256"])
    s, bufs, dl = vc.downscale_pyramid(dbuf, (nx, ny, nz), c["method"], c["alpha"], levels)
    assert s == vc.VC_OK
    for b, d, want in zip(bufs, dl, c["level_sha256"]):
        assert sha(b.download(d[0] * d[1] * d[2])) == want
        b.free()
    s, data = vc.encode_ds(vol, c["target"], c["method"], c["alpha"])
    assert s == vc.VC_OK and hashlib.sha256(data).hexdigest() == c["sha256"], name
    s, data2 = vc.encode_ds(dbuf, c["target"], c["method"], c["alpha"], on_device=(nx, ny, nz))
    assert s == vc.VC_OK and data2 == data
    if c["method"] == vc.DS_BOX:   # the codec's own pyramid
        s, plain = vc.encode(vol, c["target"])
        assert plain == data
    dbuf.free()
