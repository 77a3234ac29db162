"""Whole-atom integer DCT (vcg_dct_forward / vcg_dct_inverse): both forms, the
CUDA-core butterfly and the int8 tensor-core (IMMA) form, give the oracle's
coefficients and reconstructed voxels bit for bit, for synthetic, random and
extreme volumes, several centre values, and inverse inputs that push the IMMA
form's pieces out of range (handed back to the butterfly)."""
import ctypes

import numpy as np
import pytest

import oraclelib as O

FORMS = [0, 1]   # butterfly, imma


def atoms_of(vol):
    nz, ny, nx = vol.shape
    for az in range(nz // 32):
        for ay in range(ny // 32):
            for ax in range(nx // 32):
                yield vol[az * 32:az * 32 + 32, ay * 32:ay * 32 + 32, ax * 32:ax * 32 + 32]


def oracle_fdct(vol, centre):
    out = []
    for a in atoms_of(vol):
        v = np.ascontiguousarray(a)
        c = np.zeros(32768, np.int32)
        O.lib().orc_fdct(v.ctypes.data, centre, c.ctypes.data)
        out.append(c)
    return np.concatenate(out)


def oracle_idct(coef, dims, centre):
    nx, ny, nz = dims
    vol = np.zeros((nz, ny, nx), np.uint8)
    i = 0
    for az in range(nz // 32):
        for ay in range(ny // 32):
            for ax in range(nx // 32):
                c = np.ascontiguousarray(coef[i * 32768:(i + 1) * 32768])
                v = np.zeros(32768, np.uint8)
                O.lib().orc_idct(c.ctypes.data, centre, v.ctypes.data)
                vol[az * 32:az * 32 + 32, ay * 32:ay * 32 + 32, ax * 32:ax * 32 + 32] = v.reshape(32, 32, 32)
                i += 1
    return vol


def volumes(vc):
    rng = np.random.default_rng(31)
    yield "synth", vc.synth(64, 96, 64, vc.config_seed(3))
    yield "random", rng.integers(0, 256, (64, 32, 96), dtype=np.uint8)
    yield "zeros", np.zeros((32, 32, 32), np.uint8)
    yield "full", np.full((32, 32, 64), 255, np.uint8)
    z, y, x = np.indices((32, 64, 32))
    yield "checker", (((x + y + z) & 1) * 255).astype(np.uint8)
    yield "ramp", ((x * 8 + y * 3 + z) % 256).astype(np.uint8)


def run_forward(vc, vol, centre, form):
    nz, ny, nx = vol.shape
    dv = vc.DeviceBuffer(vol.nbytes)
    dv.upload(vol)
    dc = vc.DeviceBuffer(vol.size * 4)
    s, redone = vc.dct_forward(dv, (nx, ny, nz), centre, form, dc)
    assert s == vc.VC_OK, vc.last_error()
    assert redone == 0
    return dc.download(vol.size * 4).view(np.int32)


def run_inverse(vc, coef, dims, centre, form):
    nx, ny, nz = dims
    dc = vc.DeviceBuffer(coef.nbytes)
    dc.upload(coef)
    dv = vc.DeviceBuffer(nx * ny * nz)
    s, redone = vc.dct_inverse(dc, dims, centre, form, dv)
    assert s == vc.VC_OK, vc.last_error()
    return dv.download(nx * ny * nz).reshape(nz, ny, nx), redone


@pytest.mark.gpu
@pytest.mark.parametrize("form", FORMS)
def test_forward_and_inverse_match_oracle(vc, gpu, form):
    for name, vol in volumes(vc):
        nz, ny, nx = vol.shape
        for centre in (128, 0, 255, 37):
            ref = oracle_fdct(vol, centre)
            got = run_forward(vc, vol, centre, form)
            assert np.array_equal(got, ref), (name, centre, form)
            rec_ref = oracle_idct(ref, (nx, ny, nz), centre)
            rec, redone = run_inverse(vc, ref, (nx, ny, nz), centre, form)
            assert redone == 0
            assert np.array_equal(rec, rec_ref), (name, centre, form)


@pytest.mark.gpu
@pytest.mark.parametrize("form", FORMS)
def test_inverse_of_arbitrary_coefficients(vc, gpu, form):
    """Dequantised-like and arbitrary coefficient fields, including values whose
    intermediates overflow the IMMA pieces (and wrap the i32 sums)."""
    rng = np.random.default_rng(32)
    dims = (64, 32, 32)
    n = 2 * 32768
    cases = {
        "small": rng.integers(-300, 301, n).astype(np.int32),
        "medium": rng.integers(-(1 << 15), 1 << 15, n).astype(np.int32),
        "sparse_large": np.where(rng.random(n) < 0.01, rng.integers(-(1 << 20), 1 << 20, n), 0).astype(np.int32),
        "huge": rng.integers(-(1 << 30), 1 << 30, n).astype(np.int32),
    }
    for name, coef in cases.items():
        ref = oracle_idct(coef, dims, 128)
        got, redone = run_inverse(vc, coef, dims, 128, form)
        assert np.array_equal(got, ref), (name, form)
        if form == 1 and name == "huge":
            assert redone == 2   # both atoms handed to the butterfly
        if form == 0:
            assert redone == 0


@pytest.mark.gpu
def test_forms_agree_on_benchmark_volume_slab(vc, gpu):
    """A 256x256x64 slab of the synthetic benchmark volume: both forms identical
    and equal to the oracle on every atom."""
    vol = vc.synth(256, 256, 64, vc.config_seed(2))
    f0 = run_forward(vc, vol, 128, 0)
    f1 = run_forward(vc, vol, 128, 1)
    assert np.array_equal(f0, f1)
    assert np.array_equal(f0, oracle_fdct(vol, 128))
    r0, _ = run_inverse(vc, f0, (256, 256, 64), 128, 0)
    r1, _ = run_inverse(vc, f0, (256, 256, 64), 128, 1)
    assert np.array_equal(r0, r1)
    assert np.array_equal(r0, oracle_idct(f0, (256, 256, 64), 128))


def test_dct_argument_checks(vc):
    """Shapes that are not whole atoms, bad centres or forms and null pointers
    are VC_ERR_RANGE before any device work (no GPU needed)."""
    L = vc.lib()
    p = ctypes.c_void_p(16)
    for dims, centre, form in [((33, 32, 32), 128, 0), ((32, 32, 0), 128, 0), ((32, 32, 32), 256, 0),
                               ((32, 32, 32), -1, 1), ((32, 32, 32), 128, 2)]:
        assert L.vcg_dct_forward(p, vc.Dims(*dims), centre, form, p, None) == vc.VC_ERR_RANGE
        assert L.vcg_dct_inverse(p, vc.Dims(*dims), centre, form, p, None) == vc.VC_ERR_RANGE
    assert L.vcg_dct_forward(None, vc.Dims(32, 32, 32), 128, 0, p, None) == vc.VC_ERR_RANGE
    assert L.vcg_dct_forward(ctypes.c_void_p(17), vc.Dims(32, 32, 32), 128, 0, p, None) == vc.VC_ERR_RANGE
