"""Drive the reference codec (oracle/_ref/libvcref.so, built from the reference
source by oracle/Makefile) through its own public API.

``ref_encode`` composes the reference's writer exactly as the canonical
``vc_encode`` is defined for this project: LOD pyramid from
``vc_test_downsample2x`` (src/vc/vc.c:1562), per-LOD ``base_q`` from the
present-atom bisection measured with ``vc_test_atom_rt`` (src/vc/vc.c:1582),
then ``vc_create`` / ``vc_set_base_q`` / ``vc_append_atom`` (every atom of
every LOD in raster order, one thread) / ``vc_writer_close``.

Test infrastructure only: it exists where the reference checkout exists (the
development container), never on the GPU host.
"""
import ctypes
import os
import struct
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libvcref.so")


class Dims(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_uint32), ("ny", ctypes.c_uint32), ("nz", ctypes.c_uint32)]


class Box(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in ("x0", "y0", "z0", "x1", "y1", "z1")]


def available():
    return os.path.exists(REF_SO)


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(REF_SO)
        L.vc_create.restype = ctypes.c_void_p
        L.vc_create.argtypes = [ctypes.c_char_p, Dims, ctypes.c_float]
        L.vc_set_base_q.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float]
        L.vc_append_atom.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32,
                                     ctypes.c_uint32, ctypes.c_void_p]
        L.vc_mark_zero_atom.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32,
                                        ctypes.c_uint32]
        L.vc_mark_zero_region.argtypes = L.vc_mark_zero_atom.argtypes
        L.vc_writer_close.argtypes = [ctypes.c_void_p]
        L.vc_open.restype = ctypes.c_void_p
        L.vc_open.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        L.vc_open_streaming.restype = ctypes.c_void_p
        L.vc_open_streaming.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
        L.vc_close.argtypes = [ctypes.c_void_p]
        L.vc_lod_dims.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Dims)]
        L.vc_decode_atom.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_void_p]
        L.vc_decode_region.argtypes = [ctypes.c_void_p, ctypes.c_int, Box, ctypes.c_void_p]
        L.vc_atom_coverage.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_uint32]
        L.vc_test_atom_rt.restype = ctypes.c_uint32
        L.vc_test_atom_rt.argtypes = [ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p]
        L.vc_test_downsample2x.restype = ctypes.c_void_p
        L.vc_test_downsample2x.argtypes = [ctypes.c_void_p, Dims, ctypes.POINTER(Dims)]
        _lib = L
    return _lib


_libc = ctypes.CDLL(None)
_libc.free.argtypes = [ctypes.c_void_p]


def nlod_of(nx, ny, nz):
    n = 1
    d = (nx, ny, nz)
    for l in range(1, 8):
        d = tuple((v + 1) // 2 for v in d)
        n = l + 1
        if max(d) <= 1:
            break
    return n


def lod_dims(nx, ny, nz, lod):
    d = (nx, ny, nz)
    for _ in range(lod):
        d = tuple((v + 1) // 2 for v in d)
    return d


def downsample(vol):
    """vol: (nz, ny, nx) u8 -> next LOD via the reference's vc_test_downsample2x."""
    L = lib()
    nz, ny, nx = vol.shape
    vol = np.ascontiguousarray(vol)
    od = Dims()
    p = L.vc_test_downsample2x(vol.ctypes.data, Dims(nx, ny, nz), ctypes.byref(od))
    out = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint8)), (od.nz * od.ny * od.nx,)).copy()
    _libc.free(p)
    return out.reshape(od.nz, od.ny, od.nx)


def atoms_of(vol):
    """(nz,ny,nx) -> (acz, acy, acx, 32, 32, 32) zero-padded atom grid, raster order."""
    nz, ny, nx = vol.shape
    acz, acy, acx = (nz + 31) // 32, (ny + 31) // 32, (nx + 31) // 32
    pad = np.zeros((acz * 32, acy * 32, acx * 32), np.uint8)
    pad[:nz, :ny, :nx] = vol
    return pad.reshape(acz, 32, acy, 32, acx, 32).transpose(0, 2, 4, 1, 3, 5)


def atom_sizes(atoms, q, threads=8):
    L = lib()
    flat = [np.ascontiguousarray(a) for a in atoms.reshape(-1, 32, 32, 32)]

    def one(a):
        return L.vc_test_atom_rt(a.ctypes.data, ctypes.c_float(q), None)

    with ThreadPoolExecutor(threads) as ex:
        return np.array(list(ex.map(one, flat)), np.uint64)


def f32_bits(x):
    return struct.unpack("<I", struct.pack("<f", x))[0]


def bits_f32(b):
    return struct.unpack("<f", struct.pack("<I", b))[0]


def rate_control(vol, target, threads=8):
    """Present-atom bisection over float bit patterns in [0.05, 4096] (24 steps)."""
    atoms = atoms_of(vol).reshape(-1, 32, 32, 32)
    present = atoms.reshape(atoms.shape[0], -1).any(axis=1)
    return rate_control_atoms(atoms[present], target, threads)


def rate_control_atoms(pa, target, threads=8):
    """rate_control on the present atoms already gathered, (N, 32, 32, 32) u8."""
    npres = int(pa.shape[0])
    if npres == 0:
        return 1.0, 0, 0
    target = float(np.float32(target))
    lo, hi = f32_bits(0.05), f32_bits(4096.0)
    best_q, best_err, best_bytes = 1.0, float("inf"), 0
    for _ in range(24):
        mid = lo + (hi - lo) // 2
        q = bits_f32(mid)
        nbytes = int(atom_sizes(pa, q, threads).sum())
        ratio = (32768.0 * npres) / float(nbytes)
        err = abs(ratio - target)
        if err < best_err or (err == best_err and q > best_q):
            best_q, best_err, best_bytes = q, err, nbytes
        if ratio < target:
            lo = mid
        else:
            hi = mid
    return best_q, npres, best_bytes


def lod_qs(q0, nlod):
    qs, q = [], np.float32(q0)
    for _ in range(nlod):
        qs.append(float(max(q, np.float32(0.05))))
        q = np.float32(q * np.float32(0.6))
    return qs


def write_archive(lods, dims, target, qs, only_lod0=False, skip=(), zero_marks=()):
    """Write with the reference writer in canonical order; returns archive bytes."""
    L = lib()
    nx, ny, nz = dims
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "a.vca").encode()
        w = L.vc_create(path, Dims(nx, ny, nz), ctypes.c_float(target))
        assert w, "vc_create"
        for l, q in enumerate(qs):
            L.vc_set_base_q(w, l, ctypes.c_float(q))
        for l, vol in enumerate(lods):
            if only_lod0 and l > 0:
                break
            at = atoms_of(vol)
            acz, acy, acx = at.shape[:3]
            for az in range(acz):
                for ay in range(acy):
                    for ax in range(acx):
                        if (l, az, ay, ax) in skip:
                            continue
                        if (l, az, ay, ax) in zero_marks:
                            assert L.vc_mark_zero_atom(w, l, az, ay, ax) == 0
                            continue
                        a = np.ascontiguousarray(at[az, ay, ax])
                        assert L.vc_append_atom(w, l, az, ay, ax, a.ctypes.data) == 0
        L.vc_writer_close(w)
        with open(path, "rb") as f:
            return f.read()


def pyramid(vol):
    nz, ny, nx = vol.shape
    lods = [vol]
    for _ in range(1, nlod_of(nx, ny, nz)):
        lods.append(downsample(lods[-1]))
    return lods


def ref_encode(vol, target, threads=8):
    """The canonical vc_encode composed from reference calls. Returns (bytes, q0)."""
    nz, ny, nx = vol.shape
    lods = pyramid(vol)
    q0, _, _ = rate_control(vol, target, threads)
    qs = lod_qs(q0, len(lods))
    return write_archive(lods, (nx, ny, nz), target, qs), q0


class RefArchive:
    def __init__(self, data):
        self.buf = ctypes.create_string_buffer(bytes(data), len(data))
        self.h = lib().vc_open(ctypes.addressof(self.buf), len(data))

    def close(self):
        if self.h:
            lib().vc_close(self.h)
            self.h = None

    def lod_dims(self, lod):
        d = Dims()
        s = lib().vc_lod_dims(self.h, lod, ctypes.byref(d))
        return s, (d.nx, d.ny, d.nz)

    def decode_atom(self, lod, ax, ay, az):
        out = np.zeros(32768, np.uint8)
        s = lib().vc_decode_atom(self.h, lod, ax, ay, az, out.ctypes.data)
        return s, out

    def decode_region(self, lod, box):
        x0, y0, z0, x1, y1, z1 = box
        out = np.zeros(max(0, (x1 - x0) * (y1 - y0) * (z1 - z0)), np.uint8)
        s = lib().vc_decode_region(self.h, lod, Box(*box), out.ctypes.data)
        return s, out

    def decode_lod(self, lod):
        s, (nx, ny, nz) = self.lod_dims(lod)
        if s:
            return s, None
        s, out = self.decode_region(lod, (0, 0, 0, nx, ny, nz))
        return s, out.reshape(nz, ny, nx)

    def coverage(self, lod, az, ay, ax):
        return lib().vc_atom_coverage(self.h, lod, az, ay, ax)


READ_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p)


class RefStreamingArchive(RefArchive):
    """The reference's vc_open_streaming over read(off, n) -> n bytes, or None
    for a failed read (returned to the reference as VC_ERR_FORMAT)."""

    def __init__(self, read, total_len):
        def cb(ud, off, n, dst):
            b = read(off, n)
            if b is None or len(b) != n:
                return 1
            ctypes.memmove(dst, bytes(b), n)
            return 0
        self._cb = READ_FN(cb)
        self.h = lib().vc_open_streaming(ctypes.cast(self._cb, ctypes.c_void_p), None, total_len)


DS_SO = os.path.join(ROOT, "oracle", "_ref", "libdsref.so")
_ds = None


def ds_downscale2x(vol, method, alpha):
    """The reference exporter's ds_downscale2x (tools/downscale.h) on a (nz, ny, nx) volume."""
    global _ds
    if _ds is None:
        _ds = ctypes.CDLL(DS_SO)
        _ds.dsref_downscale2x.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_int)] * 3 + \
                                         [ctypes.c_int, ctypes.c_float]
        _ds.dsref_cell.restype = ctypes.c_uint
        _ds.dsref_cell.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float]
    vol = np.ascontiguousarray(vol, np.uint8)
    nz, ny, nx = vol.shape
    out = np.zeros(((nz + 1) // 2, (ny + 1) // 2, (nx + 1) // 2), np.uint8)
    o = [ctypes.c_int() for _ in range(3)]
    _ds.dsref_downscale2x(vol.ctypes.data, nx, ny, nz, out.ctypes.data, *[ctypes.byref(v) for v in o], method,
                          ctypes.c_float(alpha))
    assert (o[0].value, o[1].value, o[2].value) == (out.shape[2], out.shape[1], out.shape[0])
    return out


def ds_cell(c8, method, alpha):
    ds_downscale2x(np.zeros((1, 1, 1), np.uint8), 0, 0.0)   # loads the library
    c8 = np.ascontiguousarray(c8, np.uint8)
    return _ds.dsref_cell(c8.ctypes.data, method, ctypes.c_float(alpha))


def ds_encode(vol, target, method, alpha, threads=8):
    """vc_encode with the exporter's pyramid, composed from reference calls:
    levels by ds_downscale2x, q0 by the present-atom bisection on LOD 0, the
    writer in canonical order. Returns (bytes, q0, levels)."""
    nz, ny, nx = vol.shape
    lods = [vol]
    for _ in range(1, nlod_of(nx, ny, nz)):
        lods.append(ds_downscale2x(lods[-1], method, alpha))
    q0, _, _ = rate_control(vol, target, threads)
    return write_archive(lods, (nx, ny, nz), target, lod_qs(q0, len(lods))), q0, lods
