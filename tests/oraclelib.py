"""ctypes binding of the CPU oracle (oracle/liboracle.so) for the tests and the
CPU-baseline leg of bench.py. Test infrastructure only."""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "liboracle.so")


class Dims(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_uint32), ("ny", ctypes.c_uint32), ("nz", ctypes.c_uint32)]


class Box(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in ("x0", "y0", "z0", "x1", "y1", "z1")]


_lib = None
P = ctypes.c_void_p


def build():
    subprocess.check_call(["make", "-s", "-C", ORACLE_DIR, "liboracle.so"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = ctypes.CDLL(ORACLE_SO)
        L.orc_encode_atom.restype = ctypes.c_uint32
        L.orc_encode_atom.argtypes = [P, ctypes.c_float, P, ctypes.c_uint32, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_uint8)]
        L.orc_decode_atom_payload.argtypes = [P, ctypes.c_uint32, ctypes.c_float, P]
        L.orc_enc_levels.restype = ctypes.c_uint32
        L.orc_enc_levels.argtypes = [P, P, ctypes.c_uint32]
        L.orc_rc_size.restype = ctypes.c_uint32
        L.orc_rc_size.argtypes = [P]
        L.orc_dec_levels.argtypes = [P, ctypes.c_uint32, P]
        L.orc_fdct.argtypes = [P, ctypes.c_int32, P]
        L.orc_idct.argtypes = [P, ctypes.c_int32, P]
        L.orc_quantize.argtypes = [P, ctypes.c_float, P]
        L.orc_dequantize.argtypes = [P, ctypes.c_float, P]
        L.orc_dq_tables.argtypes = [ctypes.c_float, P, P]
        L.orc_tables.argtypes = [P, P, P]
        L.orc_downsample2x.argtypes = [P, Dims, P]
        L.orc_rate_control.restype = ctypes.c_float
        L.orc_rate_control.argtypes = [P, Dims, ctypes.c_float, ctypes.c_int, ctypes.POINTER(ctypes.c_uint64),
                                       ctypes.POINTER(ctypes.c_uint64)]
        L.orc_encode.argtypes = [P, Dims, ctypes.c_float, ctypes.c_int, ctypes.POINTER(P),
                                 ctypes.POINTER(ctypes.c_size_t)]
        L.orc_encode_fixed_q.argtypes = [P, Dims, ctypes.c_float, P, ctypes.c_int, ctypes.POINTER(P),
                                         ctypes.POINTER(ctypes.c_size_t)]
        L.orc_free.argtypes = [P]
        L.orc_open.restype = P
        L.orc_open.argtypes = [P, ctypes.c_size_t]
        L.orc_open_streaming.restype = P
        L.orc_ds_cell.restype = ctypes.c_uint8
        L.orc_ds_cell.argtypes = [P, ctypes.c_int, ctypes.c_float]
        L.orc_ds_downscale2x.argtypes = [P, Dims, ctypes.c_int, ctypes.c_float, P, ctypes.POINTER(Dims)]
        L.orc_ds_set_fused.argtypes = [ctypes.c_int]
        L.orc_open_streaming.argtypes = [P, P, ctypes.c_uint64]
        L.orc_close.argtypes = [P]
        L.orc_lod_dims.argtypes = [P, ctypes.c_int, ctypes.POINTER(Dims)]
        L.orc_decode_atom.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
        L.orc_decode_region.argtypes = [P, ctypes.c_int, Box, P]
        L.orc_decode_lod.argtypes = [P, ctypes.c_int, P, ctypes.POINTER(Dims)]
        L.orc_decode_lod_mt.argtypes = [P, ctypes.c_int, P, ctypes.c_int]
        L.orc_atom_coverage.argtypes = [P, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
        L.orc_atom_payload_range.argtypes = [P, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                             ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32)]
        L.orc_archive_version.argtypes = [P]
        L.orc_nlod_of.argtypes = [P]
        L.orc_base_q.restype = ctypes.c_float
        L.orc_base_q.argtypes = [P, ctypes.c_int]
        L.orc_encode_sizes_mt.restype = ctypes.c_uint64
        L.orc_encode_sizes_mt.argtypes = [P, Dims, ctypes.c_float, P, ctypes.c_uint32, P, ctypes.c_int]
        _lib = L
    return _lib


def ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def encode(vol, target, threads=8):
    """Canonical vc_encode on the CPU: returns archive bytes."""
    nz, ny, nx = vol.shape
    vol = np.ascontiguousarray(vol)
    out, n = P(), ctypes.c_size_t()
    s = lib().orc_encode(ptr(vol), Dims(nx, ny, nz), ctypes.c_float(target), threads, ctypes.byref(out),
                         ctypes.byref(n))
    if s:
        return s, None
    data = ctypes.string_at(out, n.value)
    lib().orc_free(out)
    return 0, data


def encode_fixed_q(vol, target, qs, threads=8):
    nz, ny, nx = vol.shape
    vol = np.ascontiguousarray(vol)
    qa = np.array(list(qs) + [0.0] * (8 - len(qs)), np.float32)
    out, n = P(), ctypes.c_size_t()
    s = lib().orc_encode_fixed_q(ptr(vol), Dims(nx, ny, nz), ctypes.c_float(target), ptr(qa), threads,
                                 ctypes.byref(out), ctypes.byref(n))
    if s:
        return s, None
    data = ctypes.string_at(out, n.value)
    lib().orc_free(out)
    return 0, data


def rate_control(vol, target, threads=8):
    nz, ny, nx = vol.shape
    vol = np.ascontiguousarray(vol)
    npres, nbytes = ctypes.c_uint64(), ctypes.c_uint64()
    q = lib().orc_rate_control(ptr(vol), Dims(nx, ny, nz), ctypes.c_float(target), threads,
                               ctypes.byref(npres), ctypes.byref(nbytes))
    return q, npres.value, nbytes.value


def downsample(vol):
    nz, ny, nx = vol.shape
    out = np.zeros(((nz + 1) // 2, (ny + 1) // 2, (nx + 1) // 2), np.uint8)
    lib().orc_downsample2x(ptr(np.ascontiguousarray(vol)), Dims(nx, ny, nz), ptr(out))
    return out


class Archive:
    def __init__(self, data):
        self.buf = ctypes.create_string_buffer(bytes(data), len(data))
        self.h = lib().orc_open(ctypes.addressof(self.buf), len(data))

    def close(self):
        if self.h:
            lib().orc_close(self.h)
            self.h = None

    @property
    def nlod(self):
        return lib().orc_nlod_of(self.h)

    def base_q(self, lod):
        return lib().orc_base_q(self.h, lod)

    def lod_dims(self, lod):
        d = Dims()
        s = lib().orc_lod_dims(self.h, lod, ctypes.byref(d))
        return s, (d.nx, d.ny, d.nz)

    def decode_atom(self, lod, ax, ay, az):
        out = np.zeros(32768, np.uint8)
        s = lib().orc_decode_atom(self.h, lod, ax, ay, az, ptr(out))
        return s, out

    def decode_region(self, lod, box, out=None):
        x0, y0, z0, x1, y1, z1 = box
        if out is None:
            out = np.zeros(max(0, (x1 - x0) * (y1 - y0) * (z1 - z0)), np.uint8)
        s = lib().orc_decode_region(self.h, lod, Box(*box), ptr(out))
        return s, out

    def decode_lod(self, lod, threads=0):
        s, (nx, ny, nz) = self.lod_dims(lod)
        if s:
            return s, None
        out = np.zeros((nz, ny, nx), np.uint8)
        if threads:
            s = lib().orc_decode_lod_mt(self.h, lod, ptr(out), threads)
        else:
            d = Dims()
            s = lib().orc_decode_lod(self.h, lod, ptr(out), ctypes.byref(d))
        return s, out

    def coverage(self, lod, az, ay, ax):
        return lib().orc_atom_coverage(self.h, lod, az, ay, ax)

    def payload_range(self, lod, az, ay, ax):
        o, l = ctypes.c_uint64(), ctypes.c_uint32()
        c = lib().orc_atom_payload_range(self.h, lod, az, ay, ax, ctypes.byref(o), ctypes.byref(l))
        return c, o.value, l.value
READ_FN = ctypes.CFUNCTYPE(ctypes.c_int, P, ctypes.c_uint64, ctypes.c_uint32, P)


class StreamingArchive(Archive):
    """orc_open_streaming over read(off, n) -> n bytes, or None for a failed read."""

    def __init__(self, read, total_len):
        def cb(ud, off, n, dst):
            b = read(off, n)
            if b is None or len(b) != n:
                return 1
            ctypes.memmove(dst, bytes(b), n)
            return 0
        self._cb = READ_FN(cb)
        self.h = lib().orc_open_streaming(ctypes.cast(self._cb, P), None, total_len)


def ds_downscale2x(vol, method, alpha):
    """The oracle's exporter downscale of a (nz, ny, nx) volume."""
    vol = np.ascontiguousarray(vol, np.uint8)
    nz, ny, nx = vol.shape
    out = np.zeros(((nz + 1) // 2, (ny + 1) // 2, (nx + 1) // 2), np.uint8)
    od = Dims()
    lib().orc_ds_downscale2x(ptr(vol), Dims(nx, ny, nz), method, ctypes.c_float(alpha), ptr(out), ctypes.byref(od))
    return out
