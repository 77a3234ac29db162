"""C-ABI boundary checks that need no GPU: the library loads, exports every
symbol the public headers declare, and its host-side archive handling
(header validation, coverage, payload ranges, argument checks) matches the
oracle on the golden archives. No call here reaches the device."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_archive


def header_functions(path):
    txt = open(path).read()
    txt = re.sub(r"//[^\n]*", "", txt)
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"typedef[^;]*\(\s*\*[^;]*;", "", txt)   # function-pointer types
    names = set(re.findall(r"\b(vcg?_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_headers_declare_the_reference_reader_api():
    names = header_functions(os.path.join(ROOT, "include", "vc.h"))
    for n in ["vc_encode", "vc_open", "vc_open_streaming", "vc_close", "vc_lod_dims", "vc_decode_lod", "vc_decode_atom",
              "vc_decode_region", "vc_atom_coverage", "vc_atom_payload_range", "vc_archive_version"]:
        assert n in names


def test_library_exports_every_declared_symbol(vc):
    lib_path = vc.LIB_PATH
    out = subprocess.check_output(["nm", "-D", "--defined-only", lib_path]).decode()
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    declared = []
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            declared += header_functions(os.path.join(ROOT, "include", h))
    missing = [n for n in declared if n not in exported]
    assert not missing, f"declared but not exported: {missing}"
    L = vc.lib()
    for n in declared:
        assert getattr(L, n) is not None
    # nothing but the public vc_/vcg_ surface leaks out
    assert all(n.startswith(("vc_", "vcg_")) for n in exported), sorted(exported)


def _hdr(data):
    return bytearray(data[:128]) + bytearray(data[128:])


@pytest.mark.parametrize("field,value", [
    (0, 0x12345678),            # magic
    (4, 3),                     # version
    (8, 16),                    # atom edge
    (12, 2),                    # layout (v1)
    (16, 16),                   # region atoms
    (20, 0),                    # nlod 0
    (20, 9),                    # nlod > 8
])
def test_open_rejects_bad_header(vc, oracle, golden, field, value):
    data = bytearray(load_archive(golden["synth_64_t10"]))
    data[field:field + 4] = value.to_bytes(4, "little")
    a = vc.Archive(bytes(data))
    o = oracle.Archive(bytes(data))
    assert not a and not o.h


@pytest.mark.parametrize("cap", [0, 3, 1 << 40])
def test_open_rejects_bad_l1(vc, oracle, golden, cap):
    data = bytearray(load_archive(golden["synth_64_t10"]))
    data[40:48] = cap.to_bytes(8, "little")
    assert not vc.Archive(bytes(data))
    assert not oracle.Archive(bytes(data)).h


def test_open_rejects_short_buffers(vc, golden):
    data = load_archive(golden["synth_64_t10"])
    assert not vc.Archive(data[:127])
    L = vc.lib()
    assert not L.vc_open(None, 1000)
    L.vc_close(None)


@pytest.mark.parametrize("name", ["synth_64_t10", "synth_prime_97x131x65_t20", "ref_test_basic", "tiny_1x1x1",
                                  "extreme_zero", "extreme_line"])
def test_metadata_matches_oracle(vc, oracle, golden, name):
    data = load_archive(golden[name])
    a, o = vc.Archive(data), oracle.Archive(data)
    assert a and o.h
    assert a.version() == 1
    for lod in range(o.nlod):
        assert a.lod_dims(lod) == o.lod_dims(lod)
        s, (nx, ny, nz) = o.lod_dims(lod)
        for az in range((nz + 31) // 32 + 1):
            for ay in range((ny + 31) // 32 + 1):
                for ax in range((nx + 31) // 32 + 1):
                    assert a.coverage(lod, az, ay, ax) == o.coverage(lod, az, ay, ax)
                    assert a.payload_range(lod, az, ay, ax) == o.payload_range(lod, az, ay, ax)
    assert a.lod_dims(o.nlod)[0] == vc.VC_ERR_RANGE
    assert a.lod_dims(-1)[0] == vc.VC_ERR_RANGE


def test_argument_validation_needs_no_device(vc, golden):
    data = load_archive(golden["synth_64_t10"])
    a = vc.Archive(data)
    assert a.decode_atom(0, 2, 0, 0)[0] == vc.VC_ERR_RANGE     # 64^3 -> 2 atoms per axis
    assert a.decode_atom(0, 0, 0, -1)[0] == vc.VC_ERR_RANGE
    assert a.decode_atom(9, 0, 0, 0)[0] == vc.VC_ERR_RANGE
    assert a.decode_region(0, (0, 0, 0, 65, 1, 1))[0] == vc.VC_ERR_RANGE
    assert a.decode_region(0, (3, 0, 0, 3, 1, 1))[0] == vc.VC_ERR_RANGE
    assert a.decode_region(-1, (0, 0, 0, 1, 1, 1))[0] == vc.VC_ERR_RANGE
    L = vc.lib()
    out = ctypes.c_void_p()
    n = ctypes.c_size_t()
    vol = np.zeros(8, np.uint8)
    for dims, t in [((0, 2, 2), 10.0), ((2, 2, 2), 0.5), ((2, 2, 2), float("nan")), ((1 << 21, 1, 1), 10.0)]:
        s = L.vc_encode(vc.ptr(vol), vc.Dims(*dims), ctypes.c_float(t), ctypes.byref(out), ctypes.byref(n))
        assert s == vc.VC_ERR_RANGE
    assert L.vc_region_atoms() == 32


@pytest.mark.parametrize("name", ["synth_prime_97x131x65_t20", "ref_test_basic", "synth_flat_96x64x33_t100",
                                  "tiny_1x1x1"])
def test_request_validation_matches_oracle(vc, oracle, golden, name):
    """Every region, atom and LOD request the oracle rejects as out of range
    (src/vc/vc.c:1404-1421, 1535-1555: LOD outside the archive, atom outside
    the LOD, empty box, box past the LOD's edge) is rejected by the library
    with VC_ERR_RANGE before it needs a device, and no other: with no device a
    request the oracle accepts gets VC_ERR_IO (on a GPU it would be decoded).
    Where the reference's build exists, its answers equal the oracle's."""
    import refcodec
    data = load_archive(golden[name])
    a, o = vc.Archive(data), oracle.Archive(data)
    r = refcodec.RefArchive(data) if refcodec.available() else None   # the reference's own build, this host only
    rng = np.random.default_rng(0xA46)
    edge = [0, 1, 2, 31, 32, 33, 63, 64, 96, 97, 98, 130, 131, 132, 2047, 2048, 2049, 0xFFFFFFFF, 0x80000000]

    def coord(hi):
        return int(rng.choice(edge)) if rng.integers(0, 3) == 0 else int(rng.integers(0, hi + 3))

    ranged = accepted = 0
    for _ in range(400):
        lod = int(rng.choice([-1, 0, 0, 1, 2, o.nlod - 1, o.nlod, 8, 9]))
        s, dims = o.lod_dims(lod) if 0 <= lod < o.nlod else (0, (4, 4, 4))
        lo, hi = [], []
        for d in dims:   # a valid extent on most axes, edge and random values on the others
            if rng.integers(0, 100) < 85:
                x0 = int(rng.integers(0, d))
                lo.append(x0)
                hi.append(int(rng.integers(x0 + 1, d + 1)))
            else:
                lo.append(coord(d))
                hi.append(coord(d))
        box = (lo[0], lo[1], lo[2], hi[0], hi[1], hi[2])
        n = (box[3] - box[0]) * (box[4] - box[1]) * (box[5] - box[2]) if box[3] > box[0] and box[4] > box[1] \
            and box[5] > box[2] else 0
        # a box larger than the whole LOD cannot be valid: both must refuse it before writing
        out = np.zeros(n if 0 < n <= dims[0] * dims[1] * dims[2] else 1, np.uint8)
        so = oracle.lib().orc_decode_region(o.h, lod, oracle.Box(*box), out.ctypes.data)
        sa = vc.lib().vc_decode_region(a.h, lod, vc.Box(*box), out.ctypes.data)
        assert (sa == vc.VC_ERR_RANGE) == (so == vc.VC_ERR_RANGE), (lod, box, sa, so)
        if r is not None:
            sr = refcodec.lib().vc_decode_region(r.h, lod, refcodec.Box(*box), out.ctypes.data)
            assert (sr == vc.VC_ERR_RANGE) == (so == vc.VC_ERR_RANGE), ("oracle against the reference", lod, box)
        ranged += so == vc.VC_ERR_RANGE
        accepted += so != vc.VC_ERR_RANGE
        ax, ay, az = (coord((d + 31) // 32) for d in dims)
        s1, _ = a.decode_atom(lod, ax, ay, az)
        s2, _ = o.decode_atom(lod, ax, ay, az)
        assert (s1 == vc.VC_ERR_RANGE) == (s2 == vc.VC_ERR_RANGE), (lod, ax, ay, az, s1, s2)
        if r is not None:
            s3, _ = r.decode_atom(lod, ax, ay, az)
            assert (s3 == vc.VC_ERR_RANGE) == (s2 == vc.VC_ERR_RANGE), ("oracle against the reference", lod, ax, ay, az)
    assert ranged > 50 and accepted > 20
