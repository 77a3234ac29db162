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


def atom_dc(a):
    return (int(a.astype(np.int64).sum()) + 16384) // 32768   # src/vc/vc.c:603


def oracle_fdct(vol, centre):
    """Coefficients of every atom, and the per-atom centres used (centre -1:
    each atom's dc)."""
    out, dcs = [], []
    for a in atoms_of(vol):
        v = np.ascontiguousarray(a)
        c = np.zeros(32768, np.int32)
        dc = atom_dc(v) if centre < 0 else centre
        O.lib().orc_fdct(v.ctypes.data, dc, c.ctypes.data)
        out.append(c)
        dcs.append(dc)
    return np.concatenate(out), np.array(dcs, np.uint8)


def oracle_idct(coef, dims, centre, dcs=None):
    nx, ny, nz = dims
    vol = np.zeros((nz, ny, nx), np.uint8)
    i = 0
    for az in range(nz // 32):
        for ay in range(ny // 32):
            for ax in range(nx // 32):
                c = np.ascontiguousarray(coef[i * 32768:(i + 1) * 32768])
                v = np.zeros(32768, np.uint8)
                O.lib().orc_idct(c.ctypes.data, int(dcs[i]) if centre < 0 else centre, v.ctypes.data)
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
    dcoef = vc.DeviceBuffer(vol.size * 4)
    ddc = vc.DeviceBuffer(vol.size // 32768)
    s, redone = vc.dct_forward(dv, (nx, ny, nz), centre, form, dcoef, ddc)
    assert s == vc.VC_OK, vc.last_error()
    assert redone == 0
    dcs = ddc.download(vol.size // 32768) if centre < 0 else None
    return dcoef.download(vol.size * 4).view(np.int32), dcs


def run_inverse(vc, coef, dims, centre, form, dcs=None):
    nx, ny, nz = dims
    dcoef = vc.DeviceBuffer(coef.nbytes)
    dcoef.upload(coef)
    ddc = None
    if centre < 0:
        ddc = vc.DeviceBuffer(len(dcs))
        ddc.upload(dcs)
    dv = vc.DeviceBuffer(nx * ny * nz)
    s, redone = vc.dct_inverse(dcoef, dims, centre, form, dv, ddc)
    assert s == vc.VC_OK, vc.last_error()
    return dv.download(nx * ny * nz).reshape(nz, ny, nx), redone


@pytest.mark.gpu
@pytest.mark.parametrize("form", FORMS)
def test_forward_and_inverse_match_oracle(vc, gpu, form):
    for name, vol in volumes(vc):
        nz, ny, nx = vol.shape
        for centre in (-1, 128, 0, 255, 37):   # -1: each atom's dc, as the codec centres
            ref, ref_dc = oracle_fdct(vol, centre)
            got, got_dc = run_forward(vc, vol, centre, form)
            assert np.array_equal(got, ref), (name, centre, form)
            if centre < 0:
                assert np.array_equal(got_dc, ref_dc), (name, form)
            rec_ref = oracle_idct(ref, (nx, ny, nz), centre, ref_dc)
            rec, redone = run_inverse(vc, ref, (nx, ny, nz), centre, form, ref_dc)
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
    f0, d0 = run_forward(vc, vol, -1, 0)
    f1, d1 = run_forward(vc, vol, -1, 1)
    assert np.array_equal(f0, f1) and np.array_equal(d0, d1)
    ref, ref_dc = oracle_fdct(vol, -1)
    assert np.array_equal(f0, ref) and np.array_equal(d0, ref_dc)
    r0, _ = run_inverse(vc, f0, (256, 256, 64), -1, 0, d0)
    r1, _ = run_inverse(vc, f0, (256, 256, 64), -1, 1, d0)
    assert np.array_equal(r0, r1)
    assert np.array_equal(r0, oracle_idct(f0, (256, 256, 64), -1, d0))


def test_dct_argument_checks(vc):
    """Shapes that are not whole atoms, bad centres or forms and null pointers
    are VC_ERR_RANGE before any device work (no GPU needed)."""
    L = vc.lib()
    p = ctypes.c_void_p(16)
    for dims, centre, form in [((33, 32, 32), 128, 0), ((32, 32, 0), 128, 0), ((32, 32, 32), 256, 0),
                               ((32, 32, 32), -2, 1), ((32, 32, 32), 128, 2), ((32, 32, 32), -1, 0)]:
        assert L.vcg_dct_forward(p, vc.Dims(*dims), centre, form, p, None, None) == vc.VC_ERR_RANGE
        assert L.vcg_dct_inverse(p, None, vc.Dims(*dims), centre, form, p, None) == vc.VC_ERR_RANGE
    assert L.vcg_dct_forward(None, vc.Dims(32, 32, 32), 128, 0, p, None, None) == vc.VC_ERR_RANGE
    assert L.vcg_dct_forward(ctypes.c_void_p(17), vc.Dims(32, 32, 32), 128, 0, p, None, None) == vc.VC_ERR_RANGE
