#!/usr/bin/env python3
"""Generate the golden fixtures from the reference codec (development host only).

Every archive and decoded hash here is produced by the reference's own code
(oracle/_ref/libvcref.so, built from the reference source with its release
flags) through refcodec.py; the inputs come from the seeded synthetic
generator (volume-compressor_gb300/libvcsynth.so) or from the content the
reference's own tests use (tests/test_vc.c, tests/test_coverage.c).

Output: tests/golden/golden.json (+ small archives as *.vca.xz).
    python tests/golden/gen_golden.py            # standard set (~1 min)
    python tests/golden/gen_golden.py --big      # + 1024^3 config at targets 10/50/100 (~15 min)
    python tests/golden/gen_golden.py --cfg4 --append   # + the 2048x2048x1536 t20 archive
                                                        #   and its first region boxes (~30 min)
    python tests/golden/gen_golden.py --cfg5 --append   # + the 2048^3 t20 archive and a
                                                        #   served request mix (~40 min)
"""
import hashlib
import json
import lzma
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "volume-compressor_gb300"))
import refcodec as R  # noqa: E402
import vc_gb300 as V  # noqa: E402

OUT = os.path.join(HERE, "golden.json")


def sha(b):
    return hashlib.sha256(bytes(b)).hexdigest()


def make_atom_volume(dims):
    """Content of tests/test_vc.c:34-39 (make_atom) over a whole volume."""
    nx, ny, nz = dims
    acx, acy, acz = (nx + 31) // 32, (ny + 31) // 32, (nz + 31) // 32
    z = np.arange(acz * 32)[:, None, None]
    y = np.arange(acy * 32)[None, :, None]
    x = np.arange(acx * 32)[None, None, :]
    v = 128 + 60 * np.sin(x * 0.06) + 40 * np.cos(y * 0.05) + 20 * np.sin(z * 0.07)
    return v.astype(np.uint8)   # C cast truncates toward zero; values are in [8, 248]


def decoded_hashes(data, boxes=()):
    a = R.RefArchive(data)
    nlod = int.from_bytes(data[20:24], "little")
    nx, ny, nz = (int.from_bytes(data[o:o + 4], "little") for o in (24, 28, 32))
    lods, atoms = [], []
    for lod in range(nlod):
        s, vol = a.decode_lod(lod)
        assert s == 0
        lods.append(sha(vol))
        dx, dy, dz = R.lod_dims(nx, ny, nz, lod)
        h = hashlib.sha256()
        for az in range((dz + 31) // 32):
            for ay in range((dy + 31) // 32):
                for ax in range((dx + 31) // 32):
                    s, at = a.decode_atom(lod, ax, ay, az)
                    assert s == 0
                    h.update(at.tobytes())
        atoms.append(h.hexdigest())
    regs = []
    for lod, box in boxes:
        s, out = a.decode_region(lod, box)
        regs.append({"lod": lod, "box": list(box), "status": s, "sha256": sha(out) if s == 0 else None})
    cov = []
    a.close()
    return {"lod_sha256": lods, "atoms_sha256": atoms, "regions": regs, "coverage": cov}


def random_boxes(dims, nlod, n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        lod = int(rng.integers(0, min(nlod, 3)))
        d = R.lod_dims(*dims, lod)
        box = []
        lo, hi = [], []
        for k in range(3):
            e = int(rng.integers(1, min(d[k], 90) + 1))
            o = int(rng.integers(0, d[k] - e + 1))
            lo.append(o)
            hi.append(o + e)
        out.append((lod, (lo[0], lo[1], lo[2], hi[0], hi[1], hi[2])))
    return out


def store(name, data):
    path = os.path.join(HERE, name + ".vca.xz")
    with open(path, "wb") as f:
        f.write(lzma.compress(data, preset=9))
    return os.path.basename(path)


def synth_case(name, dims, seed, target, keep=True, nboxes=6):
    nx, ny, nz = dims
    vol = V.synth(nx, ny, nz, seed)
    data, q0 = R.ref_encode(vol, target)
    nlod = R.nlod_of(*dims)
    case = {"name": name, "kind": "synth", "dims": list(dims), "seed": seed, "target": target, "q0": q0,
            "nlod": nlod, "len": len(data), "sha256": sha(data), "volume_sha256": sha(vol)}
    case.update(decoded_hashes(data, random_boxes(dims, nlod, nboxes, seed)))
    if keep:
        case["file"] = store(name, data)
    print(f"{name}: q0={q0} len={len(data)}", flush=True)
    return case


def fixed_q_case(name, dims, seed, qs):
    nx, ny, nz = dims
    vol = V.synth(nx, ny, nz, seed)
    lods = R.pyramid(vol)
    res = []
    for q in qs:
        data = R.write_archive(lods, dims, 10.0, [q] * len(lods))
        res.append({"q": q, "len": len(data), "sha256": sha(data),
                    "lod0_sha256": decoded_hashes(data)["lod_sha256"][0]})
        print(f"{name} q={q}: len={len(data)}", flush=True)
    return {"name": name, "kind": "fixed_q", "dims": list(dims), "seed": seed, "runs": res}


def writer_case(name, dims, vol, q, skip=(), zero_marks=()):
    """Archive written by the reference writer with LOD0 only (partial coverage)."""
    nx, ny, nz = dims
    lods = [vol[:nz, :ny, :nx]]
    nlod = R.nlod_of(*dims)
    data = R.write_archive(lods, dims, 30.0, [q] * nlod, only_lod0=True, skip=set(skip), zero_marks=set(zero_marks))
    a = R.RefArchive(data)
    acx, acy, acz = (nx + 31) // 32, (ny + 31) // 32, (nz + 31) // 32
    atoms, cov = [], []
    for az in range(acz):
        for ay in range(acy):
            for ax in range(acx):
                s, at = a.decode_atom(0, ax, ay, az)
                atoms.append(sha(at))
                cov.append(a.coverage(0, az, ay, ax))
    s, full = a.decode_lod(0)
    a.close()
    print(f"{name}: len={len(data)}", flush=True)
    return {"name": name, "kind": "writer", "dims": list(dims), "q": q, "len": len(data), "sha256": sha(data),
            "file": store(name, data), "atom_sha256": atoms, "coverage": cov, "lod0_sha256": sha(full),
            "skip": [list(s) for s in skip], "zero_marks": [list(z) for z in zero_marks]}


def config4_boxes(dims, nlod, n, seed=0xB0C5):
    """The batched-decode box list of the 2048x2048x1536 workload: LOD U{0..3},
    edges U[32,256] clamped to the LOD, offsets U[0, dim - edge] (numpy
    default_rng; bench.py draws the same sequence)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        lod = int(rng.integers(0, 4))
        d = R.lod_dims(*dims, lod)
        e = [int(min(rng.integers(32, 257), d[k])) for k in range(3)]
        o = [int(rng.integers(0, d[k] - e[k] + 1)) for k in range(3)]
        out.append((lod, (o[0], o[1], o[2], o[0] + e[0], o[1] + e[1], o[2] + e[2])))
    return out


def config4_case(n_boxes=400):
    """2048x2048x1536 at target_ratio 20 (the batched / served workload): the
    archive's hash and the reference's decode of the first n_boxes boxes."""
    dims = (2048, 2048, 1536)
    seed = V.config_seed(4)
    vol = V.synth(*dims, seed, threads=os.cpu_count())
    data, q0 = R.ref_encode(vol, 20.0, threads=os.cpu_count())
    vsha = sha(vol)
    del vol
    nlod = R.nlod_of(*dims)
    a = R.RefArchive(data)
    boxes = []
    for lod, box in config4_boxes(dims, nlod, n_boxes):
        s, out = a.decode_region(lod, box)
        assert s == 0
        boxes.append({"lod": lod, "box": list(box), "sha256": sha(out)})
    a.close()
    print(f"cfg4: q0={q0} len={len(data)}", flush=True)
    return {"name": "cfg4_2048x2048x1536_t20", "kind": "synth", "dims": list(dims), "seed": seed, "target": 20.0,
            "q0": q0, "nlod": nlod, "len": len(data), "sha256": sha(data), "volume_sha256": vsha,
            "box_seed": 0xB0C5, "boxes": boxes}


def served_mix(dims, n, seed=0xC5C5):
    """The served-decode request mix over the 2048^3 archive: 70% one 32^3 atom
    at LOD0, 25% boxes with edges U[64,128] at LOD 0-1, 5% 512^3 boxes at LOD2
    (numpy default_rng; bench.py draws the same sequence from this seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        u = rng.random()
        if u < 0.70:
            d = R.lod_dims(*dims, 0)
            o = [32 * int(rng.integers(0, (d[k] + 31) // 32)) for k in range(3)]
            e = [min(32, d[k] - o[k]) for k in range(3)]
            lod = 0
        elif u < 0.95:
            lod = int(rng.integers(0, 2))
            d = R.lod_dims(*dims, lod)
            e = [int(min(rng.integers(64, 129), d[k])) for k in range(3)]
            o = [int(rng.integers(0, d[k] - e[k] + 1)) for k in range(3)]
        else:
            lod = 2
            d = R.lod_dims(*dims, 2)
            e = [min(512, d[k]) for k in range(3)]
            o = [int(rng.integers(0, d[k] - e[k] + 1)) for k in range(3)]
        out.append((lod, (o[0], o[1], o[2], o[0] + e[0], o[1] + e[1], o[2] + e[2])))
    return out


def present_atoms(vol):
    """The atoms of a volume whose dims are multiples of 32 that hold a nonzero
    voxel, (N, 32, 32, 32) in raster order, gathered one atom layer at a time
    (memory: the volume plus the present atoms)."""
    nz, ny, nx = vol.shape
    acy, acx = ny // 32, nx // 32

    def layer(az):
        return np.ascontiguousarray(
            vol[az * 32:az * 32 + 32].reshape(32, acy, 32, acx, 32).transpose(1, 3, 0, 2, 4)).reshape(-1, 32, 32, 32)

    counts = [int(layer(az).reshape(acy * acx, -1).any(axis=1).sum()) for az in range(nz // 32)]
    pa = np.empty((sum(counts), 32, 32, 32), np.uint8)
    k = 0
    for az in range(nz // 32):
        a = layer(az)
        a = a[a.reshape(a.shape[0], -1).any(axis=1)]
        pa[k:k + a.shape[0]] = a
        k += a.shape[0]
    return pa


def config5_case(n_reqs=200):
    """2048^3 at target_ratio 20 (the served workload): the archive's hash and
    the reference's decode of n_reqs requests of the served mix. The volume is
    generated in slabs and the rate control gathers the present atoms once
    (refcodec.rate_control's rule, rate_control_atoms), so that the host needs
    about twice the volume in memory, not four times."""
    dims = (2048, 2048, 2048)
    nx, ny, nz = dims
    seed = V.config_seed(5)
    vol = np.empty((nz, ny, nx), np.uint8)
    for z0 in range(0, nz, 128):
        vol[z0:z0 + 128] = V.synth(nx, ny, nz, seed, threads=os.cpu_count(), z0=z0, z1=min(nz, z0 + 128))
    print("cfg5: volume", flush=True)
    lods = R.pyramid(vol)
    pa = present_atoms(vol)
    q0, _, _ = R.rate_control_atoms(pa, 20.0, threads=os.cpu_count())
    del pa
    print(f"cfg5: q0={q0}", flush=True)
    data = R.write_archive(lods, dims, 20.0, R.lod_qs(q0, len(lods)))
    del lods
    vsha = sha(vol)
    del vol
    nlod = R.nlod_of(*dims)
    a = R.RefArchive(data)
    reqs = []
    for lod, box in served_mix(dims, n_reqs):
        s, out = a.decode_region(lod, box)
        assert s == 0
        reqs.append({"lod": lod, "box": list(box), "sha256": sha(out)})
    a.close()
    print(f"cfg5: q0={q0} len={len(data)}", flush=True)
    return {"name": "cfg5_2048_t20", "kind": "synth", "dims": list(dims), "seed": seed, "target": 20.0,
            "q0": q0, "nlod": nlod, "len": len(data), "sha256": sha(data), "volume_sha256": vsha,
            "mix_seed": 0xC5C5, "requests": reqs}


def main():
    big = "--big" in sys.argv
    cases = json.load(open(OUT))["cases"] if os.path.exists(OUT) and "--append" in sys.argv else []
    names = {c["name"] for c in cases}

    def add(c):
        cases[:] = [x for x in cases if x["name"] != c["name"]] + [c]

    if "--cfg4" in sys.argv:
        add(config4_case())
    elif "--cfg5" in sys.argv:
        add(config5_case())
    elif not big or "cfg1_256_t10" not in names:
        add(synth_case("cfg1_256_t10", (256, 256, 256), V.config_seed(1), 10.0, keep=False, nboxes=10))
        add(synth_case("synth_64_t10", (64, 64, 64), 0x5EED1001, 10.0))
        add(synth_case("synth_prime_97x131x65_t20", (97, 131, 65), 0x5EED1002, 20.0))
        add(synth_case("synth_thin_2048x32x32_t50", (2048, 32, 32), 0x5EED1003, 50.0, keep=False))
        add(synth_case("synth_flat_96x64x33_t100", (96, 64, 33), 0x5EED1004, 100.0))
        # single voxel volume (nlod = 2, src/vc/vc.c:1001-1006)
        one = np.full((1, 1, 1), 77, np.uint8)
        data, q0 = R.ref_encode(one, 10.0)
        c = {"name": "tiny_1x1x1", "kind": "volume", "dims": [1, 1, 1], "value": 77, "target": 10.0, "q0": q0,
             "len": len(data), "sha256": sha(data), "file": store("tiny_1x1x1", data)}
        c.update(decoded_hashes(data))
        add(c)
        add(fixed_q_case("fixed_q_128", (128, 128, 128), 0x5EED1005,
                         [0.05, 0.3, 1.0, 2.5, 7.25, 64.0, 4096.0]))
        # reference test content: tests/test_vc.c:46-101 (ABSENT + KNOWN_ZERO atoms)
        d = (256, 192, 160)
        add(writer_case("ref_test_basic", d, make_atom_volume(d), 1.0, skip=[(0, 0, 0, 0)],
                        zero_marks=[(0, (160 + 31) // 32 - 1, 0, 0)]))
        # tests/test_coverage.c:192-255 content extremes (one atom, q = 1)
        z = np.zeros((64, 64, 64), np.uint8)
        add(writer_case("extreme_zero", (64, 64, 64), z, 1.0))
        v = z.copy(); v[5, 5, 5] = 200
        add(writer_case("extreme_voxel", (64, 64, 64), v, 1.0))
        v = z.copy(); v[5, 5, 5:13] = 200
        add(writer_case("extreme_line", (64, 64, 64), v, 1.0))
        add(writer_case("extreme_sat", (64, 64, 64), np.full((64, 64, 64), 255, np.uint8), 1.0))
    if big:
        for t in (10.0, 50.0, 100.0):
            add(synth_case(f"cfg2_1024_t{int(t)}", (1024, 1024, 1024), V.config_seed(2), t, keep=False, nboxes=6))
    json.dump({"generator": "tests/golden/gen_golden.py", "reference_build": "oracle/_ref/libvcref.so (release flags)",
               "cases": cases}, open(OUT, "w"), indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
