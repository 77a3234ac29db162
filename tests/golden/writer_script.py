"""Writer session scripts (the vc.h writer API) and their execution on a
writer library: the reference's (gen_writer.py, development host) or this
project's (tests/test_writer.py). An op is a JSON list:

  ["create", [nx, ny, nz], ratio]          ["q", lod, q]
  ["atom", lod, az, ay, ax, src]           ["box", lod, [x0, y0, z0, x1, y1, z1], src]
  ["zatom", lod, az, ay, ax]               ["zregion", lod, rz, ry, rx]
  ["cov", lod, az, ay, ax]                 ["dec", lod, az, ay, ax]
  ["dec8", lod, az0, ay0, ax0]             ["close"]

Atom / box contents (src): ["vol", l, saz, say, sax] the atom at (saz, say,
sax) of level l of the session's volume pyramid (zero outside it);
["vol", l] for a box: its own voxels of level l; ["zero"]; ["const", v];
["noise", seed, hi] uniform bytes in [0, hi) from numpy's seeded generator.
The pyramid is built with the codec's downsample rule (src/vc/vc.c:1562-1577)
from the seeded synthetic volume ["volume", [nx, ny, nz], seed].
Each op's result is a status, or [status, sha256] / [status, any, sha256]
for the reads, or [length, sha256] for close."""
import ctypes
import hashlib
import os
import tempfile

import numpy as np


class Dims(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_uint32), ("ny", ctypes.c_uint32), ("nz", ctypes.c_uint32)]


class Box(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in ("x0", "y0", "z0", "x1", "y1", "z1")]


def bind(L):
    P = ctypes.c_void_p
    L.vc_create.restype = P
    L.vc_create.argtypes = [ctypes.c_char_p, Dims, ctypes.c_float]
    L.vc_set_base_q.argtypes = [P, ctypes.c_int, ctypes.c_float]
    u = ctypes.c_uint32
    L.vc_append_atom.argtypes = [P, ctypes.c_int, u, u, u, P]
    L.vc_append_box.argtypes = [P, ctypes.c_int, Box, P]
    L.vc_mark_zero_atom.argtypes = [P, ctypes.c_int, u, u, u]
    L.vc_mark_zero_region.argtypes = [P, ctypes.c_int, u, u, u]
    L.vc_writer_decode_atom.argtypes = [P, ctypes.c_int, u, u, u, P]
    L.vc_writer_coverage.argtypes = [P, ctypes.c_int, u, u, u]
    L.vc_writer_decode_2x2x2.argtypes = [P, ctypes.c_int, u, u, u, P, ctypes.POINTER(ctypes.c_int)]
    L.vc_writer_close.argtypes = [P]
    if hasattr(L, "vcg_writer_flush"):
        L.vcg_append_atom_async.argtypes = [P, ctypes.c_int, u, u, u, P]
        L.vcg_writer_flush.argtypes = [P, ctypes.POINTER(ctypes.c_uint64)]
    return L


def downsample(v):
    """src/vc/vc.c:1562-1577: integer mean of the in-bounds 2x2x2 children."""
    nz, ny, nx = v.shape
    p = np.zeros((nz + nz % 2, ny + ny % 2, nx + nx % 2), np.int64)
    c = np.zeros_like(p)
    p[:nz, :ny, :nx] = v
    c[:nz, :ny, :nx] = 1
    s = sum(p[dz::2, dy::2, dx::2] for dz in (0, 1) for dy in (0, 1) for dx in (0, 1))
    n = sum(c[dz::2, dy::2, dx::2] for dz in (0, 1) for dy in (0, 1) for dx in (0, 1))
    return ((s + n // 2) // n).astype(np.uint8)


def pyramid(vol, nlod=8):
    lv = [vol]
    while len(lv) < nlod and max(lv[-1].shape) > 1:
        lv.append(downsample(lv[-1]))
    return lv


def region_of(level, x0, y0, z0, x1, y1, z1):
    out = np.zeros((z1 - z0, y1 - y0, x1 - x0), np.uint8)
    nz, ny, nx = level.shape
    cz, cy, cx = min(z1, nz), min(y1, ny), min(x1, nx)
    if cz > z0 and cy > y0 and cx > x0:
        out[: cz - z0, : cy - y0, : cx - x0] = level[z0:cz, y0:cy, x0:cx]
    return out


def content(src, pyr, box=None):
    kind = src[0]
    if kind == "vol":
        lv = pyr[src[1]]
        if box is not None:
            x0, y0, z0, x1, y1, z1 = box
            return region_of(lv, x0, y0, z0, x1, y1, z1)
        az, ay, ax = src[2], src[3], src[4]
        return region_of(lv, ax * 32, ay * 32, az * 32, ax * 32 + 32, ay * 32 + 32, az * 32 + 32)
    shape = (32, 32, 32) if box is None else (box[5] - box[2], box[4] - box[1], box[3] - box[0])
    if kind == "zero":
        return np.zeros(shape, np.uint8)
    if kind == "const":
        return np.full(shape, src[1], np.uint8)
    if kind == "noise":
        return np.random.default_rng(src[1]).integers(0, src[2], shape, dtype=np.uint8)
    raise ValueError(src)


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


def run(L, session, synth, async_atoms=False):
    """Execute session {"volume": [[nx, ny, nz], seed], "ops": [...]} on writer
    library L (bound with bind()); synth(nx, ny, nz, seed) makes the volume.
    Returns the list of results. With async_atoms, atom appends go through
    vcg_append_atom_async (this project's library only) and every other op
    first flushes (the flush's status is appended to the result list as
    ["flush", status, failed] when it is not clean)."""
    (nx, ny, nz), seed = session["volume"]
    pyr = pyramid(synth(nx, ny, nz, seed))
    res = []
    w = None
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "w.vca")
        for op in session["ops"]:
            k = op[0]
            if async_atoms and w and k not in ("atom", "create"):
                n = ctypes.c_uint64()
                fs = L.vcg_writer_flush(w, ctypes.byref(n))
                if fs or n.value:
                    res.append(["flush", fs, n.value])
            if k == "create":
                w = L.vc_create(path.encode(), Dims(*op[1]), ctypes.c_float(op[2]))
                res.append(1 if w else 0)
            elif k == "q":
                res.append(L.vc_set_base_q(w, op[1], ctypes.c_float(op[2])))
            elif k == "atom" and async_atoms:
                a = np.ascontiguousarray(content(op[5], pyr))
                res.append(L.vcg_append_atom_async(w, op[1], op[2], op[3], op[4], a.ctypes.data))
                continue
            elif k == "atom":
                a = np.ascontiguousarray(content(op[5], pyr))
                res.append(L.vc_append_atom(w, op[1], op[2], op[3], op[4], a.ctypes.data))
            elif k == "box":
                v = np.ascontiguousarray(content(op[3], pyr, op[2]))
                res.append(L.vc_append_box(w, op[1], Box(*op[2]), v.ctypes.data))
            elif k == "zatom":
                res.append(L.vc_mark_zero_atom(w, op[1], op[2], op[3], op[4]))
            elif k == "zregion":
                res.append(L.vc_mark_zero_region(w, op[1], op[2], op[3], op[4]))
            elif k == "cov":
                res.append(L.vc_writer_coverage(w, op[1], op[2], op[3], op[4]))
            elif k == "dec":
                out = np.full(32768, 0x5A, np.uint8)
                s = L.vc_writer_decode_atom(w, op[1], op[2], op[3], op[4], out.ctypes.data)
                res.append([s, sha(out)])
            elif k == "dec8":
                out = np.full(8 * 32768, 0x5A, np.uint8)
                anyv = ctypes.c_int(-1)
                s = L.vc_writer_decode_2x2x2(w, op[1], op[2], op[3], op[4], out.ctypes.data, ctypes.byref(anyv))
                res.append([s, anyv.value, sha(out)])
            elif k == "close":
                L.vc_writer_close(w)
                w = None
                data = open(path, "rb").read()
                res.append([len(data), sha(data)])
            else:
                raise ValueError(op)
    return res
