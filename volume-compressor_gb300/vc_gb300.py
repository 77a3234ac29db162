"""Python binding (ctypes) of the GB300 volume codec's C ABI (include/vc.h,
include/vcg.h) and of the host synthetic-volume generator.

The library is the in-tree ``libvc.so`` built by ``build.py``; there is no
fallback implementation: if the library is missing, loading raises, and without
a usable CUDA device every decode / encode returns VC_ERR_IO (4).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libvc.so")
SYNTH_PATH = os.path.join(HERE, "libvcsynth.so")

VC_OK, VC_ERR_FORMAT, VC_ERR_RANGE, VC_ERR_OOM, VC_ERR_IO = 0, 1, 2, 3, 4
VC_ABSENT, VC_KNOWN_ZERO, VC_PRESENT = 0, 1, 2

# Every symbol the public headers declare (checked by the CPU test suite).
VC_SYMBOLS = ["vc_encode", "vc_open", "vc_close", "vc_lod_dims", "vc_decode_lod", "vc_decode_atom",
              "vc_decode_region", "vc_atom_coverage", "vc_atom_payload_range", "vc_archive_version",
              "vc_region_blob_range", "vc_region_atoms", "vc_set_panic_hook", "vc_open_streaming",
              "vc_create", "vc_set_base_q", "vc_append_atom", "vc_append_box", "vc_mark_zero_atom",
              "vc_mark_zero_region", "vc_writer_decode_atom", "vc_writer_coverage", "vc_writer_decode_2x2x2",
              "vc_writer_close"]
VCG_SYMBOLS = ["vcg_decode_region_device", "vcg_decode_lod_device", "vcg_make_resident", "vcg_encode_device",
               "vcg_encode_q", "vcg_decode_atoms_noalloc", "vcg_decode_regions", "vcg_batch_shape",
               "vcg_set_batch_shape", "vcg_repack_v2", "vcg_set_rc_scalar_warps", "vcg_set_rc_solo",
               "vcg_set_stream_threads", "vcg_memory_read", "vcg_downscale2x", "vcg_downscale_pyramid",
               "vcg_append_atom_async", "vcg_writer_flush",
               "vcg_encode_ds", "vcg_dct_forward", "vcg_dct_inverse",
               "vcg_server_create", "vcg_server_submit", "vcg_server_wait", "vcg_server_stats",
               "vcg_server_destroy",
               "vcg_synth_volume_device", "vcg_alloc", "vcg_free", "vcg_alloc_host", "vcg_free_host", "vcg_copy",
               "vcg_memset", "vcg_sync", "vcg_device_info", "vcg_device_memory", "vcg_debug_fail_alloc",
               "vcg_last_error", "vcg_profile_enable",
               "vcg_profile_read", "vcg_last_call_ms"]


class Dims(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_uint32), ("ny", ctypes.c_uint32), ("nz", ctypes.c_uint32)]


class Box(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in ("x0", "y0", "z0", "x1", "y1", "z1")]


class RegionRequest(ctypes.Structure):
    _fields_ = [("lod", ctypes.c_int32), ("box", Box), ("out", ctypes.c_void_p)]


class Server:
    """vcg_server_*: continuous-batching decode server over one Archive. submit()
    keeps the output array alive until wait() returns its ticket."""

    def __init__(self, archive, device_budget, max_batch, workers):
        self.archive = archive
        self.h = lib().vcg_server_create(archive.h, device_budget, max_batch, workers)
        if not self.h:
            raise RuntimeError("vcg_server_create failed")
        self._outs = {}

    def submit(self, lod, box, out):
        t = lib().vcg_server_submit(self.h, lod, Box(*box), out.ctypes.data)
        if t >= 0:
            self._outs[t] = out
        return t

    def wait(self, ticket):
        """Returns (status, latency in microseconds)."""
        lat = ctypes.c_double()
        s = lib().vcg_server_wait(self.h, ticket, ctypes.byref(lat))
        self._outs.pop(ticket, None)
        return s, lat.value

    def stats(self):
        b, r = ctypes.c_uint64(), ctypes.c_uint64()
        lib().vcg_server_stats(self.h, ctypes.byref(b), ctypes.byref(r))
        return b.value, r.value

    def close(self):
        if self.h:
            lib().vcg_server_destroy(self.h)
            self.h = None
            self._outs.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


DCT_BUTTERFLY, DCT_IMMA, DCT_ATOM_DC = 0, 1, -1


def dct_forward(vol, dims, centre, form, coef, dc=None):
    """vcg_dct_forward: vol, coef (and dc, for centre DCT_ATOM_DC) DeviceBuffers;
    dims (nx, ny, nz). Returns (status, atoms redone)."""
    r = ctypes.c_uint32()
    s = lib().vcg_dct_forward(vol.ptr, Dims(*dims), centre, form, coef.ptr, dc.ptr if dc else None,
                              ctypes.byref(r))
    return s, r.value


def dct_inverse(coef, dims, centre, form, vol, dc=None):
    """vcg_dct_inverse: coef, vol (and dc, for centre DCT_ATOM_DC) DeviceBuffers;
    dims (nx, ny, nz). Returns (status, atoms redone)."""
    r = ctypes.c_uint32()
    s = lib().vcg_dct_inverse(coef.ptr, dc.ptr if dc else None, Dims(*dims), centre, form, vol.ptr,
                              ctypes.byref(r))
    return s, r.value


def batch_shape():
    """(range-decoder policy, transform threads, transform on the tensor cores) the autotuner chose."""
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    lib().vcg_batch_shape(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
    return a.value, b.value, c.value


P = ctypes.c_void_p
_lib = None
_synth = None


def build(force=False):
    import importlib.util
    spec = importlib.util.spec_from_file_location("vc_gb300_build", os.path.join(HERE, "build.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    m.build(force=force)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is not built (run build.py); there is no fallback implementation")
        L = ctypes.CDLL(LIB_PATH)
        L.vc_encode.argtypes = [P, Dims, ctypes.c_float, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_size_t)]
        L.vc_open.restype = P
        L.vc_open.argtypes = [P, ctypes.c_size_t]
        L.vc_open_streaming.restype = P
        u32 = ctypes.c_uint32
        L.vc_create.restype = P
        L.vc_create.argtypes = [ctypes.c_char_p, Dims, ctypes.c_float]
        L.vc_set_base_q.argtypes = [P, ctypes.c_int, ctypes.c_float]
        L.vc_append_atom.argtypes = [P, ctypes.c_int, u32, u32, u32, P]
        L.vc_append_box.argtypes = [P, ctypes.c_int, Box, P]
        L.vc_mark_zero_atom.argtypes = [P, ctypes.c_int, u32, u32, u32]
        L.vc_mark_zero_region.argtypes = [P, ctypes.c_int, u32, u32, u32]
        L.vc_writer_decode_atom.argtypes = [P, ctypes.c_int, u32, u32, u32, P]
        L.vc_writer_coverage.argtypes = [P, ctypes.c_int, u32, u32, u32]
        L.vc_writer_decode_2x2x2.argtypes = [P, ctypes.c_int, u32, u32, u32, P, ctypes.POINTER(ctypes.c_int)]
        L.vc_writer_close.argtypes = [P]
        L.vcg_append_atom_async.argtypes = [P, ctypes.c_int, u32, u32, u32, P]
        L.vcg_writer_flush.argtypes = [P, ctypes.POINTER(ctypes.c_uint64)]
        L.vc_open_streaming.argtypes = [P, P, ctypes.c_uint64]
        L.vcg_set_stream_threads.argtypes = [ctypes.c_int]
        L.vcg_downscale2x.argtypes = [P, ctypes.c_int, Dims, ctypes.c_int, ctypes.c_float, P, ctypes.POINTER(Dims)]
        L.vcg_downscale_pyramid.argtypes = [P, Dims, ctypes.c_int, ctypes.c_float, ctypes.c_int, P]
        L.vcg_encode_ds.argtypes = [P, ctypes.c_int, Dims, ctypes.c_float, P, ctypes.c_int, ctypes.c_float,
                                    ctypes.POINTER(P), ctypes.POINTER(ctypes.c_size_t)]
        L.vc_close.argtypes = [P]
        L.vc_lod_dims.argtypes = [P, ctypes.c_int, ctypes.POINTER(Dims)]
        L.vc_decode_lod.argtypes = [P, ctypes.c_int, P, ctypes.POINTER(Dims)]
        L.vc_decode_atom.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
        L.vc_decode_region.argtypes = [P, ctypes.c_int, Box, P]
        L.vc_atom_coverage.argtypes = [P, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
        L.vc_atom_payload_range.argtypes = [P, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                            ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint32)]
        L.vc_archive_version.argtypes = [P]
        L.vc_region_blob_range.argtypes = [P, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                           ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
        L.vc_region_atoms.restype = ctypes.c_uint32
        L.vcg_decode_region_device.argtypes = [P, ctypes.c_int, Box, P]
        L.vcg_decode_lod_device.argtypes = [P, ctypes.c_int, P, ctypes.POINTER(Dims)]
        L.vcg_make_resident.argtypes = [P]
        L.vcg_encode_device.argtypes = [P, Dims, ctypes.c_float, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_size_t),
                                        ctypes.POINTER(ctypes.c_float)]
        L.vcg_encode_q.argtypes = [P, ctypes.c_int, Dims, ctypes.c_float, P, ctypes.POINTER(P),
                                   ctypes.POINTER(ctypes.c_size_t)]
        L.vcg_synth_volume_device.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, P]
        L.vcg_alloc.restype = P
        L.vcg_alloc.argtypes = [ctypes.c_size_t]
        L.vcg_free.argtypes = [P]
        L.vcg_alloc_host.restype = P
        L.vcg_alloc_host.argtypes = [ctypes.c_size_t]
        L.vcg_free_host.argtypes = [P]
        L.vcg_copy.argtypes = [P, P, ctypes.c_size_t]
        L.vcg_memset.argtypes = [P, ctypes.c_int, ctypes.c_size_t]
        L.vcg_device_info.argtypes = [ctypes.POINTER(ctypes.c_int)] * 3
        L.vcg_device_memory.argtypes = [ctypes.POINTER(ctypes.c_size_t)] * 2
        L.vcg_debug_fail_alloc.argtypes = [ctypes.c_int64]
        L.vcg_debug_fail_alloc.restype = ctypes.c_int64
        L.vcg_last_error.restype = ctypes.c_char_p
        L.vcg_decode_atoms_noalloc.argtypes = [P, ctypes.c_size_t, P, P, ctypes.c_uint32, ctypes.c_float, P]
        L.vcg_decode_regions.argtypes = [P, ctypes.c_uint32, P, ctypes.c_int, P]
        L.vcg_batch_shape.argtypes = [ctypes.POINTER(ctypes.c_int)] * 3
        L.vcg_set_batch_shape.argtypes = [ctypes.c_int] * 3
        L.vcg_repack_v2.argtypes = [P, ctypes.POINTER(P), ctypes.POINTER(ctypes.c_size_t)]
        L.vcg_set_rc_scalar_warps.argtypes = [ctypes.c_int]
        L.vcg_set_rc_solo.argtypes = [ctypes.c_int]
        L.vcg_dct_forward.argtypes = [P, Dims, ctypes.c_int, ctypes.c_int, P, P, ctypes.POINTER(ctypes.c_uint32)]
        L.vcg_dct_inverse.argtypes = [P, P, Dims, ctypes.c_int, ctypes.c_int, P, ctypes.POINTER(ctypes.c_uint32)]
        L.vcg_server_create.restype = P
        L.vcg_server_create.argtypes = [P, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int]
        L.vcg_server_submit.restype = ctypes.c_int64
        L.vcg_server_submit.argtypes = [P, ctypes.c_int, Box, P]
        L.vcg_server_wait.argtypes = [P, ctypes.c_int64, ctypes.POINTER(ctypes.c_double)]
        L.vcg_server_stats.argtypes = [P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
        L.vcg_server_destroy.argtypes = [P]
        L.vcg_profile_enable.argtypes = [ctypes.c_int]
        L.vcg_profile_read.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.vcg_last_call_ms.restype = ctypes.c_double
        _lib = L
    return _lib


_libc = ctypes.CDLL(None)
_libc.free.argtypes = [P]


def ptr(a):
    return a.ctypes.data_as(P)


def last_error():
    return lib().vcg_last_error().decode()


# ---------------------------------------------------------------- device memory
class DeviceBuffer:
    """A cudaMalloc'd buffer owned by Python."""

    def __init__(self, nbytes):
        self.nbytes = int(nbytes)
        self.ptr = lib().vcg_alloc(self.nbytes)
        if not self.ptr:
            raise MemoryError(f"vcg_alloc({nbytes}) failed: {last_error()}")

    def upload(self, arr):
        a = np.ascontiguousarray(arr)
        assert a.nbytes <= self.nbytes
        if lib().vcg_copy(self.ptr, ptr(a), a.nbytes):
            raise RuntimeError(last_error())

    def download(self, nbytes=None, dtype=np.uint8):
        n = self.nbytes if nbytes is None else nbytes
        out = np.empty(n, np.uint8)
        if lib().vcg_copy(ptr(out), self.ptr, n):
            raise RuntimeError(last_error())
        return out.view(dtype)

    def free(self):
        if self.ptr:
            lib().vcg_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def sync():
    return lib().vcg_sync()


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("ms", ctypes.c_double), ("launches", ctypes.c_uint64),
                ("bytes_read", ctypes.c_uint64), ("bytes_written", ctypes.c_uint64), ("units", ctypes.c_uint64)]


def profile_enable(on=True):
    lib().vcg_profile_enable(1 if on else 0)


def profile_read(reset=True):
    """Accumulated per-stage kernel statistics {name: {ms, launches, bytes_read, bytes_written, units}}."""
    arr = (KernelStat * 32)()
    n = lib().vcg_profile_read(arr, 32, 1 if reset else 0)
    return {arr[i].name.decode(): {"ms": arr[i].ms, "launches": arr[i].launches, "bytes_read": arr[i].bytes_read,
                                   "bytes_written": arr[i].bytes_written, "units": arr[i].units}
            for i in range(min(n, 32))}


def last_call_ms():
    """Device time (CUDA events on the library stream) of this thread's last decode/encode call."""
    return lib().vcg_last_call_ms()


def device_info():
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    s = lib().vcg_device_info(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
    return s, a.value, (b.value, c.value)


def device_memory():
    """(status, free bytes, total bytes) of the library's device (cudaMemGetInfo)."""
    f, t = ctypes.c_size_t(), ctypes.c_size_t()
    s = lib().vcg_device_memory(ctypes.byref(f), ctypes.byref(t))
    return s, f.value, t.value


# ---------------------------------------------------------------- codec
def encode(vol, target_ratio):
    """vc_encode: (nz, ny, nx) u8 host volume -> (status, archive bytes)."""
    vol = np.ascontiguousarray(vol, np.uint8)
    nz, ny, nx = vol.shape
    out, n = P(), ctypes.c_size_t()
    s = lib().vc_encode(ptr(vol), Dims(nx, ny, nz), ctypes.c_float(target_ratio), ctypes.byref(out), ctypes.byref(n))
    if s:
        return s, None
    data = ctypes.string_at(out, n.value)
    _libc.free(out)
    return s, data


def encode_device(dbuf, dims, target_ratio):
    """vcg_encode_device on a DeviceBuffer holding an (nz, ny, nx) volume."""
    nx, ny, nz = dims
    out, n, q0 = P(), ctypes.c_size_t(), ctypes.c_float()
    s = lib().vcg_encode_device(dbuf.ptr, Dims(nx, ny, nz), ctypes.c_float(target_ratio), ctypes.byref(out),
                                ctypes.byref(n), ctypes.byref(q0))
    if s:
        return s, None, None
    data = ctypes.string_at(out, n.value)
    _libc.free(out)
    return s, data, q0.value


DS_BOX, DS_CBOX = 0, 1


def ds_dims(dims):
    return tuple((n + 1) // 2 for n in dims)


def downscale2x(vol, method, alpha=0.5):
    """vcg_downscale2x on a host volume (nz, ny, nx): (status, level-1 array)."""
    vol = np.ascontiguousarray(vol, np.uint8)
    nz, ny, nx = vol.shape
    ox, oy, oz = ds_dims((nx, ny, nz))
    out = np.zeros((oz, oy, ox), np.uint8)
    od = Dims()
    s = lib().vcg_downscale2x(ptr(vol), 0, Dims(nx, ny, nz), method, ctypes.c_float(alpha), ptr(out), ctypes.byref(od))
    return s, out


def downscale_pyramid(dbuf, dims, method, alpha, levels):
    """vcg_downscale_pyramid of a device volume: (status, [DeviceBuffer per level], [dims per level])."""
    bufs, dl, d = [], [], tuple(dims)
    for _ in range(levels):
        d = ds_dims(d)
        dl.append(d)
        bufs.append(DeviceBuffer(max(1, d[0] * d[1] * d[2])))
    arr = (P * levels)(*[b.ptr for b in bufs])
    s = lib().vcg_downscale_pyramid(dbuf.ptr, Dims(*dims), method, ctypes.c_float(alpha), levels, arr)
    return s, bufs, dl


def encode_ds(vol, target_ratio, method, alpha=0.5, qs=None, on_device=None):
    """vcg_encode_ds: the exporter's pyramid; qs None = rate control."""
    qa = None
    if qs is not None:
        qa = np.zeros(8, np.float32)
        qa[:len(qs)] = qs
    out, n = P(), ctypes.c_size_t()
    if on_device is None:
        vol = np.ascontiguousarray(vol, np.uint8)
        nz, ny, nx = vol.shape
        src, flag = ptr(vol), 0
    else:
        nx, ny, nz = on_device
        src, flag = vol.ptr, 1
    s = lib().vcg_encode_ds(src, flag, Dims(nx, ny, nz), ctypes.c_float(target_ratio),
                            ptr(qa) if qa is not None else None, method, ctypes.c_float(alpha),
                            ctypes.byref(out), ctypes.byref(n))
    if s:
        return s, None
    data = ctypes.string_at(out, n.value)
    _libc.free(out)
    return s, data


def encode_q(vol, target_ratio, qs, on_device=None):
    """vcg_encode_q: explicit per-LOD base_q. vol: host array or DeviceBuffer (then on_device=dims)."""
    qa = np.zeros(8, np.float32)
    qa[:len(qs)] = qs
    out, n = P(), ctypes.c_size_t()
    if on_device is None:
        vol = np.ascontiguousarray(vol, np.uint8)
        nz, ny, nx = vol.shape
        s = lib().vcg_encode_q(ptr(vol), 0, Dims(nx, ny, nz), ctypes.c_float(target_ratio), ptr(qa),
                               ctypes.byref(out), ctypes.byref(n))
    else:
        nx, ny, nz = on_device
        s = lib().vcg_encode_q(vol.ptr, 1, Dims(nx, ny, nz), ctypes.c_float(target_ratio), ptr(qa),
                               ctypes.byref(out), ctypes.byref(n))
    if s:
        return s, None
    data = ctypes.string_at(out, n.value)
    _libc.free(out)
    return s, data


class Archive:
    """An opened archive (vc_open borrows the buffer, so it is kept here)."""

    def __init__(self, data):
        self.buf = ctypes.create_string_buffer(bytes(data), len(data))
        self.h = lib().vc_open(ctypes.addressof(self.buf), len(data))

    def __bool__(self):
        return bool(self.h)

    def close(self):
        if self.h:
            lib().vc_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def version(self):
        return lib().vc_archive_version(self.h)

    def lod_dims(self, lod):
        d = Dims()
        s = lib().vc_lod_dims(self.h, lod, ctypes.byref(d))
        return s, (d.nx, d.ny, d.nz)

    def make_resident(self):
        return lib().vcg_make_resident(self.h)

    def decode_atom(self, lod, ax, ay, az, out=None):
        if out is None:
            out = np.zeros(32768, np.uint8)
        s = lib().vc_decode_atom(self.h, lod, ax, ay, az, ptr(out))
        return s, out

    def decode_region(self, lod, box, out=None):
        x0, y0, z0, x1, y1, z1 = box
        if out is None:
            out = np.zeros(max(0, (x1 - x0) * (y1 - y0) * (z1 - z0)), np.uint8)
        s = lib().vc_decode_region(self.h, lod, Box(*box), ptr(out))
        return s, out

    def decode_lod(self, lod, out=None):
        s, (nx, ny, nz) = self.lod_dims(lod)
        if s:
            return s, None
        if out is None:
            out = np.zeros((nz, ny, nx), np.uint8)
        d = Dims()
        s = lib().vc_decode_lod(self.h, lod, ptr(out), ctypes.byref(d))
        return s, out

    def decode_lod_device(self, lod, dbuf):
        d = Dims()
        return lib().vcg_decode_lod_device(self.h, lod, dbuf.ptr, ctypes.byref(d))

    def decode_region_device(self, lod, box, dbuf):
        return lib().vcg_decode_region_device(self.h, lod, Box(*box), dbuf.ptr)

    def decode_regions(self, reqs, outs, on_device=False):
        """vcg_decode_regions: reqs = [(lod, (x0,y0,z0,x1,y1,z1))], outs = numpy arrays (host)
        or DeviceBuffers (device). Returns (call status, per-request statuses)."""
        arr = (RegionRequest * len(reqs))()
        for i, ((lod, box), o) in enumerate(zip(reqs, outs)):
            arr[i].lod = lod
            arr[i].box = Box(*box)
            arr[i].out = o.ptr if on_device else o.ctypes.data
        st = np.zeros(len(reqs), np.int32)
        s = lib().vcg_decode_regions(self.h, len(reqs), arr, 1 if on_device else 0, ptr(st))
        return s, st

    def repack_v2(self):
        """vcg_repack_v2: (status, v2 archive bytes)."""
        out, n = P(), ctypes.c_size_t()
        s = lib().vcg_repack_v2(self.h, ctypes.byref(out), ctypes.byref(n))
        if s:
            return s, None
        data = ctypes.string_at(out, n.value)
        _libc.free(out)
        return s, data

    def server(self, device_budget=1 << 30, max_batch=4096, workers=2):
        return Server(self, device_budget, max_batch, workers)

    def coverage(self, lod, az, ay, ax):
        return lib().vc_atom_coverage(self.h, lod, az, ay, ax)

    def payload_range(self, lod, az, ay, ax):
        o, l = ctypes.c_uint64(), ctypes.c_uint32()
        c = lib().vc_atom_payload_range(self.h, lod, az, ay, ax, ctypes.byref(o), ctypes.byref(l))
        return c, o.value, l.value


READ_FN = ctypes.CFUNCTYPE(ctypes.c_int, P, ctypes.c_uint64, ctypes.c_uint32, P)


class MemorySource(ctypes.Structure):
    _fields_ = [("buf", P), ("len", ctypes.c_uint64), ("reads", ctypes.c_uint64), ("bytes", ctypes.c_uint64)]


class StreamingArchive(Archive):
    """vc_open_streaming. `source` is either the archive bytes, served by the
    library's native vcg_memory_read, or a callable read(off, n) returning n
    bytes (None or a short result fails the read). total_len defaults to the
    length of the bytes."""

    def __init__(self, source, total_len=None):
        if callable(source):
            def cb(ud, off, n, dst):
                try:
                    b = source(off, n)
                except Exception:
                    return VC_ERR_IO
                if b is None or len(b) != n:
                    return VC_ERR_FORMAT
                ctypes.memmove(dst, bytes(b), n)
                return VC_OK
            self._cb = READ_FN(cb)
            fn, ud = ctypes.cast(self._cb, P), None
            self.src = None
        else:
            data = bytes(source)
            self.buf = ctypes.create_string_buffer(data, len(data))
            self.src = MemorySource(ctypes.addressof(self.buf), len(data), 0, 0)
            fn, ud = ctypes.cast(lib().vcg_memory_read, P), ctypes.addressof(self.src)
            if total_len is None:
                total_len = len(data)
        self.h = lib().vc_open_streaming(fn, ud, total_len)

    def reads(self):
        """(calls, bytes) served by the native memory source."""
        return (self.src.reads, self.src.bytes) if self.src is not None else None


class Writer:
    """vc_create / vc_append_* / vc_mark_zero_* / vc_writer_* / vc_writer_close."""

    def __init__(self, path, dims, target_ratio):
        self.path = path
        self.h = lib().vc_create(path.encode(), Dims(*dims), ctypes.c_float(target_ratio))

    def __bool__(self):
        return bool(self.h)

    def set_base_q(self, lod, q):
        return lib().vc_set_base_q(self.h, lod, ctypes.c_float(q))

    def append_atom(self, lod, az, ay, ax, vox):
        vox = np.ascontiguousarray(vox, np.uint8)
        return lib().vc_append_atom(self.h, lod, az, ay, ax, ptr(vox))

    def append_box(self, lod, box, voxels):
        voxels = np.ascontiguousarray(voxels, np.uint8)
        return lib().vc_append_box(self.h, lod, Box(*box), ptr(voxels))

    def append_atom_async(self, lod, az, ay, ax, vox):
        vox = np.ascontiguousarray(vox, np.uint8)
        return lib().vcg_append_atom_async(self.h, lod, az, ay, ax, ptr(vox))

    def flush(self):
        """vcg_writer_flush: (status, failed count)."""
        n = ctypes.c_uint64()
        return lib().vcg_writer_flush(self.h, ctypes.byref(n)), n.value

    def mark_zero_atom(self, lod, az, ay, ax):
        return lib().vc_mark_zero_atom(self.h, lod, az, ay, ax)

    def mark_zero_region(self, lod, rz, ry, rx):
        return lib().vc_mark_zero_region(self.h, lod, rz, ry, rx)

    def coverage(self, lod, az, ay, ax):
        return lib().vc_writer_coverage(self.h, lod, az, ay, ax)

    def decode_atom(self, lod, az, ay, ax):
        out = np.zeros(32768, np.uint8)
        return lib().vc_writer_decode_atom(self.h, lod, az, ay, ax, ptr(out)), out

    def decode_2x2x2(self, lod, az0, ay0, ax0):
        out = np.zeros((8, 32768), np.uint8)
        anyv = ctypes.c_int()
        s = lib().vc_writer_decode_2x2x2(self.h, lod, az0, ay0, ax0, ptr(out), ctypes.byref(anyv))
        return s, anyv.value, out

    def close(self):
        if self.h:
            lib().vc_writer_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def set_stream_threads(n):
    return lib().vcg_set_stream_threads(n)


# ---------------------------------------------------------------- synthetic volumes
def synth_lib():
    global _synth
    if _synth is None:
        S = ctypes.CDLL(SYNTH_PATH)
        S.vcs_cfg_size.restype = ctypes.c_size_t
        S.vcs_setup.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64]
        S.vcs_generate.argtypes = [P, P, ctypes.c_int]
        S.vcs_generate_slab.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32, P, ctypes.c_int]
        _synth = S
    return _synth


def config_seed(config_id):
    return 0x5EED0000 + config_id


def synth(nx, ny, nz, seed, threads=8, z0=0, z1=None):
    """Host-generated synthetic volume (planes [z0, z1)) as (nz, ny, nx) u8."""
    S = synth_lib()
    cfg = ctypes.create_string_buffer(S.vcs_cfg_size())
    S.vcs_setup(cfg, nx, ny, nz, seed)
    z1 = nz if z1 is None else z1
    out = np.zeros((z1 - z0, ny, nx), np.uint8)
    s = S.vcs_generate_slab(cfg, z0, z1, ptr(out), threads)
    if s:
        raise RuntimeError(f"vcs_generate_slab failed ({s})")
    return out


def synth_device(nx, ny, nz, seed):
    buf = DeviceBuffer(nx * ny * nz + 16)
    s = lib().vcg_synth_volume_device(nx, ny, nz, seed, buf.ptr)
    if s:
        raise RuntimeError(f"vcg_synth_volume_device failed ({s}): {last_error()}")
    return buf
