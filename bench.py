#!/usr/bin/env python3
"""Benchmark: LOD0 decode throughput of the 1024^3 synthetic scroll volume
encoded at target_ratio 10 (the per-atom codec path's headline workload).

GPU arm (default): the archive is produced by this library's vc_encode on the
device, opened and made resident; one step = vcg_decode_lod_device(LOD0) with
the archive and the 1 GiB output in HBM (L2 flushed between steps by a 512 MiB
write). `e2e` = one step through the drop-in C ABI with host buffers:
vc_open on a pinned host archive + vc_decode_lod into pinned host memory +
vc_close (archive upload, atom-table build, decode and copy-out all timed).

Reference arm (--impl reference): the reference's CPU decode of the same LOD0
(oracle/_ref when the reference was built on this host, else the C oracle
port), a parallel-for over atoms on all host cores.

Multi-GPU: replicas (each rank decodes its own copy; no data-path collective).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "volume-compressor_gb300")
sys.path.insert(0, PKG)

METRIC = "LOD0 decode/encode GB/s; region p50/p99 µs; bit-exact vs reference"
CONFIG_ID = 2


def args_parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--size", type=int, default=1024)
    p.add_argument("--target", type=float, default=10.0)
    p.add_argument("--regions", type=int, default=200)
    p.add_argument("--no-batched", action="store_true", help="skip the config-4 batched-region measurement")
    p.add_argument("--no-served", action="store_true", help="skip the config-5 served-decode measurement")
    p.add_argument("--no-dct", action="store_true", help="skip the config-3 DCT-forms measurement")
    p.add_argument("--no-ds", action="store_true", help="skip the exporter-downscale measurement")
    p.add_argument("--no-writer", action="store_true", help="skip the writer-append measurement")
    p.add_argument("--no-sweep", action="store_true", help="skip the config-2 target / LOD sweep")
    p.add_argument("--no-atom", action="store_true", help="skip the single-atom random-access measurement")
    p.add_argument("--dct-size", type=int, default=1024, help="edge of the DCT-forms volume")
    p.add_argument("--dct-reps", type=int, default=3, help="timed calls per DCT form and direction (0: one call)")
    p.add_argument("--detail", default=os.path.join(ROOT, "gpurun_out", "bench_detail.json"),
                   help="file that receives the full record (sweeps, batched, served, DCT, writer); '' for none")
    return p.parse_args()


def golden_named(name):
    try:
        with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
            return {c["name"]: c for c in json.load(f)["cases"]}.get(name)
    except (OSError, ValueError, KeyError):
        return None


def golden_case(size, target):
    try:
        with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
            cases = {c["name"]: c for c in json.load(f)["cases"]}
        return cases.get(f"cfg2_{size}_t{int(target)}")
    except (OSError, ValueError):
        return None


# ---------------------------------------------------------------- distributed plumbing
class Dist:
    def __init__(self):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        os.environ.setdefault("VC_DEVICE", str(self.local))
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)])
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)])
        self.pg.all_reduce(t)
        return float(t.item())


# ---------------------------------------------------------------- clocks
class Clocks:
    """SM clock and clock-event (throttle) reasons sampled during a timed region:
    NVML read-only queries every 5 ms from a thread (libnvidia-ml through
    ctypes), else nvidia-smi every 200 ms."""
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown", 0x4: "sw_power_cap",
               0x80: "hw_power_brake_slowdown"}
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.samples, self.mask, self.max_mhz = [], 0, None
        self.stop_ev = threading.Event()
        self.p = self.t = None
        self.nvml = self._nvml(gpu_index)
        if self.nvml:
            self.t = threading.Thread(target=self._loop, daemon=True)
            self.t.start()
        else:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            try:
                self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                           "-i", str(gpu_index), "-lms", "200"], stdout=self.f,
                                          stderr=subprocess.DEVNULL)
            except OSError:
                self.p = None

    def _nvml(self, idx):
        try:
            L = ctypes.CDLL("libnvidia-ml.so.1")
            if L.nvmlInit_v2() != 0:
                return None
            h = ctypes.c_void_p()
            if L.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(idx), ctypes.byref(h)) != 0:
                return None
            mx = ctypes.c_uint()
            if L.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:
                self.max_mhz = float(mx.value)
            reasons = getattr(L, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                L.nvmlDeviceGetCurrentClocksThrottleReasons
            return L, h, reasons
        except (OSError, AttributeError):
            return None

    def _loop(self):
        L, h, reasons = self.nvml
        mhz, r = ctypes.c_uint(), ctypes.c_ulonglong()
        while not self.stop_ev.is_set():
            if L.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(mhz)) == 0:
                self.samples.append(float(mhz.value))
            if reasons(h, ctypes.byref(r)) == 0:
                self.mask |= r.value
            time.sleep(0.005)

    def stop(self):
        if self.t:
            self.stop_ev.set()
            self.t.join()
            return {"sm_mhz": statistics.median(self.samples) if self.samples else None, "sm_max_mhz": self.max_mhz,
                    "reasons": sorted(n for bit, n in self.REASONS.items() if self.mask & bit),
                    "samples": len(self.samples), "source": "nvml, 5 ms"}
        if self.p:
            self.p.terminate()
            self.p.wait()
        rows = []
        if self.p:
            self.f.flush()
            with open(self.f.name) as f:
                for line in f:
                    parts = [x.strip() for x in line.split(",")]
                    if len(parts) >= 9:
                        rows.append(parts)
            os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "source": "nvidia-smi, 200 ms"}


# What bounds each decode stage, from the ncu captures of this workload (an HBM
# fraction alone misreads a latency-bound kernel).
LIMITER = {
    "decode_fused": "the range decoders' dependency chains (8 warps per SM) beside the transform's integer multiplies "
                    "(8 warps per SM) in one kernel",
    "rc_decode": "instructions and dependency chain of the per-lane range decoder (one decision per step): "
                 "ALU pipe 55 %, DRAM about 1 % busy (ncu)",
    "idct": "integer multiply-adds of the inverse passes: FMA-heavy pipe 62 % busy, 53 % of its measured IMAD "
            "rate over the transform's 1.06 M IMAD per atom; DRAM 6 % busy (ncu)",
}


def dram_traffic(kernel, units):
    """DRAM bytes (read + write) of one launch of `kernel` processing `units`
    atoms, scaled from the per-atom figure of an ncu capture committed in
    profiles/dram_traffic.json; None when there is none."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            per_atom = json.load(f)["bytes_per_atom"][kernel]
        return per_atom * units
    except (OSError, ValueError, KeyError):
        return None


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


# ---------------------------------------------------------------- CPU baseline (oracle / reference)
def cpu_decode_setup(size, target, threads):
    """Archive of the benchmark volume built on the CPU with the oracle at the
    reference's q (from the golden fixture), for the CPU arms."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oraclelib
    import vc_gb300 as vc
    g = golden_case(size, target)
    vol = vc.synth(size, size, size, vc.config_seed(CONFIG_ID), threads=threads)
    if g:
        q0 = g["q0"]
    else:
        q0, _, _ = oraclelib.rate_control(vol, target, threads)
    import numpy as np
    qs, q = [], np.float32(q0)
    for _ in range(8):
        qs.append(float(max(q, np.float32(0.05))))
        q = np.float32(q * np.float32(0.6))
    s, data = oraclelib.encode_fixed_q(vol, target, qs, threads)
    assert s == 0
    return data, q0


def host_info():
    """The host CPU (model name) and its logical core count."""
    import subprocess
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() == "Model name":
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if model is None:
        try:
            for line in open("/proc/cpuinfo"):
                if line.startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return {"cpu_model": model, "nproc": os.cpu_count()}


def cpu_one_thread(data, n_atoms=512):
    """One host thread decoding a sample of LOD0 atoms with the CPU decoder that
    cpu_decoder uses: (GB/s, kind, sample)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    ref_so = os.path.join(ROOT, "oracle", "_ref", "libvcref.so")
    if os.path.exists(ref_so):
        sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
        import refcodec
        a, kind = refcodec.RefArchive(data), "reference"
    else:
        import oraclelib
        a, kind = oraclelib.Archive(data), "port"
    _, (nx, ny, nz) = a.lod_dims(0)
    atoms = [(ax, ay, az) for az in range((nz + 31) // 32) for ay in range((ny + 31) // 32)
             for ax in range((nx + 31) // 32)]
    pick = np.random.default_rng(0x1CE).choice(len(atoms), min(n_atoms, len(atoms)), replace=False)
    t0 = time.perf_counter()
    for i in pick:
        ax, ay, az = atoms[int(i)]
        s, _ = a.decode_atom(0, ax, ay, az)
        assert s == 0
    dt = time.perf_counter() - t0
    return len(pick) * 32768 / dt / 1e9, kind, f"{len(pick)} LOD0 atoms chosen at random, one host thread"


def cpu_decoder(data, threads):
    """Returns (kind, decode_fn) timing a full LOD0 decode on the host cores."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    ref_so = os.path.join(ROOT, "oracle", "_ref", "libvcref.so")
    if os.path.exists(ref_so):
        try:
            sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
            import refcodec
            from concurrent.futures import ThreadPoolExecutor
            a = refcodec.RefArchive(data)
            _, (nx, ny, nz) = a.lod_dims(0)
            atoms = [(ax, ay, az) for az in range((nz + 31) // 32) for ay in range((ny + 31) // 32)
                     for ax in range((nx + 31) // 32)]
            L = refcodec.lib()
            bufs = [np.zeros(32768, np.uint8) for _ in range(threads)]
            out = np.zeros((nz, ny, nx), np.uint8)

            def chunk(k):
                b = bufs[k]
                for (ax, ay, az) in atoms[k::threads]:
                    L.vc_decode_atom(a.h, 0, ax, ay, az, b.ctypes.data)
                    v = b.reshape(32, 32, 32)
                    z1, y1, x1 = min(32, nz - az * 32), min(32, ny - ay * 32), min(32, nx - ax * 32)
                    out[az * 32:az * 32 + z1, ay * 32:ay * 32 + y1, ax * 32:ax * 32 + x1] = v[:z1, :y1, :x1]

            def run():
                with ThreadPoolExecutor(threads) as ex:
                    list(ex.map(chunk, range(threads)))
                return out
            return "reference", run
        except OSError:
            pass
    import oraclelib
    a = oraclelib.Archive(data)

    def run():
        s, out = a.decode_lod(0, threads=threads)
        assert s == 0
        return out
    return "port", run


def _pct(v, q):
    v = sorted(v)
    return v[min(len(v) - 1, int(q * len(v)))] if v else None


def cpu_regions(data, reqs, one_n=40, all_n=200, budget_s=8.0, check=None):
    """Per-request CPU region decode (the oracle's vc_decode_region, a scalar C
    restatement of the reference's; the reference's own build does not exist on
    this host) on a bounded sample of the same requests: one host thread in
    sequence (at most one_n requests or budget_s seconds), then all host threads
    with that many requests in flight (all_n requests). Latency per request in
    microseconds; GB/s on box bytes. `check(i, out)` (optional) sees every
    output of the all-threads pass."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    import oraclelib
    from concurrent.futures import ThreadPoolExecutor
    o = oraclelib.Archive(data)

    def one(i):
        lod, box = reqs[i]
        out = np.empty(_box_bytes(box), np.uint8)
        t0 = time.perf_counter()
        s, _ = o.decode_region(lod, box, out)
        dt = time.perf_counter() - t0
        assert s == 0
        if check:
            check(i, out)
        return dt
    lat1, t_end = [], time.perf_counter() + budget_s
    for i in range(min(one_n, len(reqs))):
        lat1.append(one(i))
        if time.perf_counter() > t_end:
            break
    n1 = len(lat1)
    b1 = sum(_box_bytes(reqs[i][1]) for i in range(n1))
    threads = os.cpu_count() or 1
    idx = list(range(min(all_n, len(reqs))))
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        latn = list(ex.map(one, idx))
    wall = time.perf_counter() - t0
    bn = sum(_box_bytes(reqs[i][1]) for i in idx)
    o.close()
    us = lambda v: [x * 1e6 for x in v]   # noqa: E731
    return {"kind": "port", "cores": threads,
            "one_thread": {"requests": n1, "p50_us": _pct(us(lat1), 0.5), "p99_us": _pct(us(lat1), 0.99),
                           "GBps": b1 / max(1e-9, sum(lat1)) / 1e9},
            "all_cores": {"requests": len(idx), "p50_us": _pct(us(latn), 0.5), "p99_us": _pct(us(latn), 0.99),
                          "GBps": bn / wall / 1e9},
            "sample": "the first requests of the same list, oracle vc_decode_region into host memory"}


def cpu_encode(vol_slab, q, one_n=256):
    """CPU encode of the atoms of a host volume slab at base_q q with the oracle's
    per-atom encoder (forward DCT, quantiser, range coder; the reference's
    vc_test_atom_rt path, src/vc/vc.c:1582-1590), all host threads over every
    atom of the slab and one thread over one_n atoms: GB/s of voxels."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    import oraclelib
    from concurrent.futures import ThreadPoolExecutor
    L = oraclelib.lib()
    z, y, x = vol_slab.shape
    atoms = np.ascontiguousarray(vol_slab.reshape(z // 32, 32, y // 32, 32, x // 32, 32)
                                 .transpose(0, 2, 4, 1, 3, 5).reshape(-1, 32768))
    threads = os.cpu_count() or 1
    import threading
    tl = threading.local()   # one payload buffer per thread

    def enc(i):
        if not hasattr(tl, "buf"):
            tl.buf = np.empty(131136, np.uint8)
        zf, dc = ctypes.c_int(), ctypes.c_uint8()
        return L.orc_encode_atom(atoms[i].ctypes.data, ctypes.c_float(q), tl.buf.ctypes.data, 131136,
                                 ctypes.byref(zf), ctypes.byref(dc))
    t0 = time.perf_counter()
    for i in range(min(one_n, len(atoms))):
        enc(i)
    t1 = time.perf_counter() - t0
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        total = sum(ex.map(enc, range(len(atoms))))
    tn = time.perf_counter() - t0
    return {"kind": "port", "cores": threads, "q": q, "atoms": len(atoms), "coder_bytes": int(total),
            "all_cores_GBps": len(atoms) * 32768 / tn / 1e9,
            "one_thread_GBps": min(one_n, len(atoms)) * 32768 / t1 / 1e9,
            "sample": f"{len(atoms)} atoms of the volume's first {z} planes, fixed q (one encode pass)"}


def config4_batched(n_boxes=10000, plain_sample=100, batch_repeats=3):
    """BASELINE config 4: 2048x2048x1536 volume at target_ratio 20; n_boxes boxes,
    edges U[32,256] (clamped to the LOD), unaligned offsets, LOD U{0..3}, seed
    0xB0C5. Batched decode (one graph replay) vs one plain decode per request,
    both into device memory; bit-exactness checked on a sample."""
    import numpy as np
    import vc_gb300 as vc
    nx, ny, nz = 2048, 2048, 1536
    dv = vc.synth_device(nx, ny, nz, vc.config_seed(4))
    s, data, q0 = vc.encode_device(dv, (nx, ny, nz), 20.0)
    assert s == 0, vc.last_error()
    dv.free()
    a = vc.Archive(data)
    assert a.make_resident() == 0
    rng = np.random.default_rng(0xB0C5)
    reqs, total = [], 0
    for _ in range(n_boxes):
        lod = int(rng.integers(0, 4))
        d = a.lod_dims(lod)[1]
        e = [int(min(rng.integers(32, 257), d[k])) for k in range(3)]
        o = [int(rng.integers(0, d[k] - e[k] + 1)) for k in range(3)]
        reqs.append((lod, (o[0], o[1], o[2], o[0] + e[0], o[1] + e[1], o[2] + e[2])))
        total += e[0] * e[1] * e[2]
    arena = vc.DeviceBuffer(total + 16 * n_boxes)

    class View:   # a request's slice of the arena
        def __init__(self, p):
            self.ptr = p
    views, off = [], 0
    for _, b in reqs:
        views.append(View(arena.ptr + off))
        off += ((b[3] - b[0]) * (b[4] - b[1]) * (b[5] - b[2]) + 15) & ~15
    ms = []
    for k in range(batch_repeats + 1):   # the first call also autotunes and captures the graph
        s, st = a.decode_regions(reqs, views, on_device=True)
        assert s == 0 and (st == 0).all()
        if k:
            ms.append(vc.last_call_ms())
    shape = vc.batch_shape()
    batch_ms = min(ms)
    # the first boxes against the reference's decode of the same archive (golden hashes)
    import hashlib
    ref_ok, ref_n = None, 0
    g = golden_named("cfg4_2048x2048x1536_t20")
    arc_ok = None if g is None else g["sha256"] == hashlib.sha256(data).hexdigest()
    if arc_ok:
        ref_ok = True
        for i, b in enumerate(g["boxes"]):
            lod, box = reqs[i]
            if (lod, list(box)) != (b["lod"], b["box"]):
                ref_ok = False
                break
            nb = (box[3] - box[0]) * (box[4] - box[1]) * (box[5] - box[2])
            host = np.empty(nb, np.uint8)
            assert vc.lib().vcg_copy(host.ctypes.data, views[i].ptr, nb) == 0
            ref_ok = ref_ok and hashlib.sha256(host.tobytes()).hexdigest() == b["sha256"]
            ref_n += 1
    elif g:
        ref_ok = False
    # every candidate of the autotuner on the same batch (forced shape, graph re-captured)
    cand = {}
    L = vc.lib()
    for rcw in (1, 4, 16):
        for tx, imma in ((256, 0), (512, 0), (256, 1)):
            assert L.vcg_set_batch_shape(rcw, tx, imma) == 0
            t = []
            for k in range(3):
                s, st = a.decode_regions(reqs, views, on_device=True)
                assert s == 0 and (st == 0).all()
                if k:
                    t.append(vc.last_call_ms())
            cand[f"rc{rcw}_{'imma' if imma else 'butterfly'}{tx}"] = min(t)
    assert L.vcg_set_batch_shape(0, 0, 0) == 0
    # the CPU's per-request decode of the first boxes, each output compared
    # with the batch's
    cpu, cpu_ok = None, [True]
    if os.environ.get("VC_BENCH_NO_CPU") != "1":
        def same(i, out):
            host = np.empty(out.size, np.uint8)
            assert vc.lib().vcg_copy(host.ctypes.data, views[i].ptr, out.size) == 0
            cpu_ok[0] = cpu_ok[0] and bool(np.array_equal(host, out))
        cpu = cpu_regions(data, reqs, one_n=40, all_n=160, check=same)
        cpu["batch_outputs_equal"] = cpu_ok[0]
    # plain path: one vcg_decode_region_device per request, on a sample
    idx = rng.choice(n_boxes, plain_sample, replace=False)
    plain_ms, plain_bytes = [], 0
    ok = True
    for i in idx:
        lod, b = reqs[i]
        nb = (b[3] - b[0]) * (b[4] - b[1]) * (b[5] - b[2])
        buf = vc.DeviceBuffer(nb)
        assert a.decode_region_device(lod, b, buf) == 0
        plain_ms.append(vc.last_call_ms())
        plain_bytes += nb
        got_plain = buf.download(nb)
        tmp = vc.DeviceBuffer(nb)
        vc.lib().vcg_copy(tmp.ptr, views[i].ptr, nb)
        ok = ok and bool(np.array_equal(tmp.download(nb), got_plain))
    plain_ms.sort()
    plain_gbps = plain_bytes / (sum(plain_ms) / 1e3) / 1e9
    batch_gbps = total / (batch_ms / 1e3) / 1e9
    return {"workload": f"{n_boxes} boxes, edges U[32,256], LOD U{{0..3}}, 2048x2048x1536 at target_ratio 20",
            "q0": q0, "archive_bytes": len(data), "box_bytes": total,
            "batched_ms": batch_ms, "batched_GBps": batch_gbps, "batched_us_per_request": batch_ms * 1e3 / n_boxes,
            "plain_GBps": plain_gbps, "plain_p50_us": plain_ms[len(plain_ms) // 2] * 1e3,
            "plain_p99_us": plain_ms[min(len(plain_ms) - 1, int(0.99 * len(plain_ms)))] * 1e3,
            "speedup_vs_plain": batch_gbps / plain_gbps, "candidates_ms": cand,
            "autotuned_shape": {"rc_scalar_warps": shape[0], "transform_imma": shape[2], "transform_threads": shape[1]},
            "bit_exact_sample": ok, "plain_sample": plain_sample,
            "bit_exact_vs_reference": {"archive": arc_ok, "boxes": ref_ok, "boxes_checked": ref_n},
            "cpu_baseline": cpu}


def _stage_table(stats, peak):
    """Per-stage device ms, algorithmic GB/s and fraction of the measured HBM peak."""
    out = {}
    for k, v in stats.items():
        gbps = (v["bytes_read"] + v["bytes_written"]) / max(1e-9, v["ms"] / 1e3) / 1e9
        out[k] = {"ms": v["ms"], "launches": v["launches"], "GBps_algorithmic": gbps, "hbm_frac": gbps / peak}
    return out


def config2_sweep(dvol, dims, peak, targets=(10.0, 50.0, 100.0)):
    """The 1024^3 volume encoded at each target (rate control included) and every
    LOD of each archive decoded into device memory: device time, GB/s and
    per-stage algorithmic GB/s with the fraction of the measured HBM peak;
    archives and decoded LODs are checked against the reference's SHA-256
    fixtures where they exist. Beside the encode, the CPU's fixed-q encode of a
    bounded sample of the same volume."""
    import hashlib
    import numpy as np
    import vc_gb300 as vc
    nx, ny, nz = dims
    res = {}
    slab = None if os.environ.get("VC_BENCH_NO_CPU") == "1" else \
        vc.synth(nx, ny, nz, vc.config_seed(CONFIG_ID), threads=os.cpu_count() or 1, z0=0, z1=min(nz, 128))
    for t in targets:
        vc.profile_enable(True)
        vc.profile_read(reset=True)
        s, data, q0 = vc.encode_device(dvol, dims, t)
        assert s == 0, vc.last_error()
        enc_ms = vc.last_call_ms()
        enc_stages = _stage_table(vc.profile_read(reset=True), peak)
        vc.profile_enable(False)
        g = golden_case(nx, t)
        row = {"q0": q0, "archive_bytes": len(data), "ratio_over_volume": nx * ny * nz / len(data),
               "encode_ms_profiled": enc_ms, "encode_stages": enc_stages,
               "archive_sha_matches_reference": (hashlib.sha256(data).hexdigest() == g["sha256"]) if g else None}
        s, _, _ = vc.encode_device(dvol, dims, t)   # unprofiled timing
        row["encode_GBps"] = nx * ny * nz / (vc.last_call_ms() / 1e3) / 1e9
        qs, qq = [], np.float32(q0)
        for _ in range(8):
            qs.append(float(max(qq, np.float32(0.05))))
            qq = np.float32(qq * np.float32(0.6))
        s, _ = vc.encode_q(dvol, t, qs, on_device=dims)
        row["encode_fixed_q_GBps"] = nx * ny * nz / (vc.last_call_ms() / 1e3) / 1e9
        if slab is not None:
            row["cpu_encode_fixed_q"] = cpu_encode(slab, q0)
        a = vc.Archive(data)
        assert a.make_resident() == 0
        lods, lod_ok = [], []
        for lod in range(8):
            s, (lx, ly, lz) = a.lod_dims(lod)
            if s:
                break
            buf = vc.DeviceBuffer(max(1, lx * ly * lz))
            assert a.decode_lod_device(lod, buf) == 0
            vc.profile_enable(True)
            vc.profile_read(reset=True)
            ms = []
            for _ in range(3):
                assert a.decode_lod_device(lod, buf) == 0
                ms.append(vc.last_call_ms())
            st = _stage_table(vc.profile_read(reset=True), peak)
            vc.profile_enable(False)
            m = statistics.median(ms)
            lods.append({"lod": lod, "dims": [lx, ly, lz], "ms": m, "GBps": lx * ly * lz / (m / 1e3) / 1e9,
                         "stages": {k: {"ms": v["ms"] / 3, "hbm_frac": v["hbm_frac"]} for k, v in st.items()}})
            if g:
                lod_ok.append(hashlib.sha256(buf.download(lx * ly * lz).tobytes()).hexdigest() == g["lod_sha256"][lod])
            buf.free()
        # the v2 container: repacked on the device, then decoded through its directory
        s, v2 = a.repack_v2()
        assert s == 0, vc.last_error()
        s, _ = a.repack_v2()
        rp_ms = vc.last_call_ms()
        a.close()
        b = vc.Archive(v2)
        assert b.make_resident() == 0
        buf = vc.DeviceBuffer(nx * ny * nz)
        assert b.decode_lod_device(0, buf) == 0
        ms = []
        for _ in range(3):
            assert b.decode_lod_device(0, buf) == 0
            ms.append(vc.last_call_ms())
        v2_ok = (hashlib.sha256(buf.download(nx * ny * nz).tobytes()).hexdigest() == g["lod_sha256"][0]) if g else None
        buf.free()
        b.close()
        row["v2"] = {"bytes": len(v2), "repack_ms": rp_ms, "repack_GBps": len(data) / (rp_ms / 1e3) / 1e9,
                     "lod0_decode_GBps": nx * ny * nz / (statistics.median(ms) / 1e3) / 1e9,
                     "lod0_matches_reference": v2_ok}
        want0 = g["lod_sha256"][0] if g else None
        row["streamed_lod0"] = {"v1": streamed_lod0(vc, data, dims, want0), "v2": streamed_lod0(vc, v2, dims, want0)}
        row["decode_lods"] = lods
        row["lods_match_reference"] = all(lod_ok) if g else None
        res[f"t{int(t)}"] = row
    return res


def atom_latency(dvol, dims, target=20.0, n=50, warm=10):
    """Random access to one 32^3 atom: the volume encoded at `target`, the
    archive resident in device memory, and n random LOD0 atoms (after `warm`
    untimed ones) decoded one call at a time through vc_decode_atom into host
    memory: wall time per call, the call's device time and its stages. Beside
    it (unless VC_BENCH_NO_CPU=1), the same atoms decoded by one host thread
    with the oracle's vc_decode_atom (a scalar C restatement of the
    reference's), whose bytes every GPU atom must equal."""
    import numpy as np
    import vc_gb300 as vc
    s, data, q0 = vc.encode_device(dvol, dims, target)
    assert s == 0, vc.last_error()
    a = vc.Archive(data)
    assert a.make_resident() == 0
    _, (lx, ly, lz) = a.lod_dims(0)
    rng = np.random.default_rng(7)
    atoms = [(int(rng.integers(0, (lx + 31) // 32)), int(rng.integers(0, (ly + 31) // 32)),
              int(rng.integers(0, (lz + 31) // 32))) for _ in range(warm + n)]
    out = np.zeros(32768, np.uint8)
    for ax, ay, az in atoms[:warm]:
        assert a.decode_atom(0, ax, ay, az, out)[0] == 0
    wall, dev, got = [], [], []
    vc.profile_enable(True)
    vc.profile_read(reset=True)
    for ax, ay, az in atoms[warm:]:
        t0 = time.perf_counter()
        s, _ = a.decode_atom(0, ax, ay, az, out)
        wall.append((time.perf_counter() - t0) * 1e3)
        assert s == 0
        dev.append(vc.last_call_ms())
        got.append(out.copy())
    st = vc.profile_read(reset=True)
    vc.profile_enable(False)
    lens = [a.payload_range(0, az, ay, ax)[2] for ax, ay, az in atoms[warm:]]
    a.close()
    res = {"target_ratio": target, "q0": q0, "atoms": n, "mean_payload_bytes": float(np.mean(lens)),
           "wall_ms_p50": _pct(wall, 0.5), "wall_ms_p99": _pct(wall, 0.99),
           "device_ms_p50": _pct(dev, 0.5),
           "stages_ms_per_call": {k: v["ms"] / n for k, v in st.items()},
           "launches_per_call": sum(v["launches"] for v in st.values()) / n}
    if os.environ.get("VC_BENCH_NO_CPU") != "1":
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oraclelib
        o = oraclelib.Archive(data)
        cpu, same = [], True
        for (ax, ay, az), g in zip(atoms[warm:], got):
            t0 = time.perf_counter()
            s, ref = o.decode_atom(0, ax, ay, az)
            cpu.append((time.perf_counter() - t0) * 1e3)
            same = same and s == 0 and np.array_equal(ref, g)
        o.close()
        res["cpu_one_thread"] = {"kind": "port", "cores": 1, "ms_p50": _pct(cpu, 0.5), "ms_p99": _pct(cpu, 0.99),
                                 "sample": "the same atoms, oracle vc_decode_atom, one host thread"}
        res["bit_exact_vs_oracle"] = bool(same)
    return res


def streamed_lod0(vc, data, dims, want, threads=(1, 8), reps=5):
    """LOD0 of `data` through vc_open_streaming: the library's memory byte
    source over the archive in pageable host memory (the stand-in for a cache of
    a remote object), payloads pulled through the callback into pinned staging
    and uploaded while the next ones are read, output to pinned host memory.
    Wall clock of vc_open_streaming + vc_decode_lod + vc_close, median of reps
    after one warm-up, per number of fetch threads."""
    import ctypes
    import hashlib
    import numpy as np
    L = vc.lib()
    nx, ny, nz = dims
    nbytes = nx * ny * nz
    src_buf = ctypes.create_string_buffer(bytes(data), len(data))
    ho = L.vcg_alloc_host(nbytes)
    out = np.ctypeslib.as_array((ctypes.c_uint8 * nbytes).from_address(ho))
    d = vc.Dims()
    res = {}
    for th in threads:
        prev = vc.set_stream_threads(th)
        ts = []
        for k in range(reps + 1):
            src = vc.MemorySource(ctypes.addressof(src_buf), len(data), 0, 0)
            t0 = time.perf_counter()
            h = L.vc_open_streaming(ctypes.cast(L.vcg_memory_read, ctypes.c_void_p), ctypes.addressof(src), len(data))
            st = L.vc_decode_lod(h, 0, ho, ctypes.byref(d))
            L.vc_close(h)
            t1 = time.perf_counter()
            assert st == 0, vc.last_error()
            if k:
                ts.append(t1 - t0)
        vc.set_stream_threads(prev)
        m = statistics.median(ts)
        res[f"threads{th}"] = {"ms": m * 1e3, "GBps": nbytes / m / 1e9, "reads": src.reads, "bytes_read": src.bytes,
                               "matches_reference": (hashlib.sha256(out).hexdigest() == want) if want else None}
    del out
    L.vcg_free_host(ho)
    return res


def _equal_device(vc, a, b, nbytes, chunk=256 << 20):
    """Byte-compare two device buffers chunk by chunk on the host."""
    import numpy as np
    ha = np.empty(min(chunk, nbytes), np.uint8)
    hb = np.empty(min(chunk, nbytes), np.uint8)
    L = vc.lib()
    for o in range(0, nbytes, chunk):
        n = min(chunk, nbytes - o)
        L.vcg_copy(ha.ctypes.data, ctypes.c_void_p(a.ptr + o), n)
        L.vcg_copy(hb.ctypes.data, ctypes.c_void_p(b.ptr + o), n)
        if not np.array_equal(ha[:n], hb[:n]):
            return False
    return True


def downscale_bench(dvol, dims, peak, reps=5, slab=64):
    """The exporter's 2x downscale (DS_BOX, and DS_CBOX at the exporter's
    alpha 0.5) of the resident 1024^3 volume: the full cascade (levels 1..7)
    and level 1 alone (the dominant launch: 1 GiB read, 128 MiB written), device
    time, algorithmic GB/s and the fraction of the measured HBM copy rate.
    Level 1 of a slab of `slab` planes is checked against the oracle, whose
    time on that slab (one host thread) is the CPU leg."""
    import numpy as np
    import vc_gb300 as vc
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oraclelib
    nx, ny, nz = dims
    levels = 7
    res = {}
    for method, name, alpha in ((vc.DS_BOX, "box", 0.5), (vc.DS_CBOX, "cbox", 0.5)):
        row = {}
        for lv in (1, levels):
            ms = []
            for r in range(reps + 1):
                s, bufs, dl = vc.downscale_pyramid(dvol, dims, method, alpha, lv)
                assert s == 0, vc.last_error()
                if r:
                    ms.append(vc.last_call_ms())
                if r < reps:
                    for b in bufs:
                        b.free()
            m = statistics.median(ms)
            dd = [tuple(dims)] + dl
            alg = sum(dd[i][0] * dd[i][1] * dd[i][2] + dd[i + 1][0] * dd[i + 1][1] * dd[i + 1][2] for i in range(lv))
            row[f"levels{lv}"] = {"ms": m, "algorithmic_bytes": alg, "GBps": alg / (m / 1e3) / 1e9,
                                  "hbm_frac": alg / (m / 1e3) / 1e9 / peak}
            if lv == 1:   # check a slab against the oracle (CPU leg)
                ox, oy = dl[0][0], dl[0][1]
                lvl1 = bufs[0].download(ox * oy * (slab // 2)).reshape(slab // 2, oy, ox)
                host = np.empty((slab, ny, nx), np.uint8)
                vc.lib().vcg_copy(host.ctypes.data, ctypes.c_void_p(dvol.ptr), host.nbytes)
                t0 = time.perf_counter()
                want = oraclelib.ds_downscale2x(host, method, alpha)
                t_cpu = time.perf_counter() - t0
                row["slab_matches_oracle"] = bool(np.array_equal(lvl1, want))
                row["cpu_port_1thread_GBps"] = host.nbytes / t_cpu / 1e9
            for b in bufs:
                b.free()
        res[name] = row
    res["note"] = ("levels1 = one launch over the 1 GiB level 0; levels7 = the cascade to 8^3; "
                   "algorithmic bytes = every level read once + its output written once")
    return res


def writer_bench(dvol, dims, q0, g, threads=16, cpu_sample=1024, sync_atoms=2048):
    """The writer API on the 1024^3 volume at the headline's LOD0 base_q: the
    whole LOD0 through one vc_append_box; through `threads` host threads
    calling vc_append_atom for every atom (each call waits for its batch: the
    concurrent calls are encoded together; timed on the first `sync_atoms`
    atoms); and through vcg_append_atom_async
    from one and from `threads` threads, then vcg_writer_flush.
    Wall clock from vc_create to vc_writer_close (file in a temporary
    directory; vc_append_box: median of 3 runs after one that sizes the
    buffers); the files must decode to the reference's LOD0. CPU leg: the
    oracle's atom encoder (transform, quantiser, coder) on `cpu_sample` atoms of
    the volume with the same number of host threads."""
    import hashlib
    import tempfile
    import threading
    import numpy as np
    import vc_gb300 as vc
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oraclelib
    nx, ny, nz = dims
    host = dvol.download(nx * ny * nz).reshape(nz, ny, nx)
    want = g["lod_sha256"][0] if g else None
    res = {"q0": q0}

    def check(path):
        a = vc.Archive(open(path, "rb").read())
        s, out = a.decode_lod(0)
        a.close()
        return (s == 0 and hashlib.sha256(out.tobytes()).hexdigest() == want) if want else None

    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "box.vca")
        ts = []
        for _ in range(4):   # the first run sizes the device and pinned buffers; median of the other 3
            t0 = time.perf_counter()
            w = vc.Writer(path, dims, 10.0)
            assert w.set_base_q(0, q0) == 0
            assert w.append_box(0, (0, 0, 0, nx, ny, nz), host) == 0
            w.close()
            ts.append(time.perf_counter() - t0)
        tb = statistics.median(ts[1:])
        res["append_box"] = {"s": tb, "GBps": nx * ny * nz / tb / 1e9, "runs_s": [round(t, 4) for t in ts[1:]],
                             "file_bytes": os.path.getsize(path), "lod0_matches_reference": check(path)}
        atoms = [(az, ay, ax) for az in range(nz // 32) for ay in range(ny // 32) for ax in range(nx // 32)]
        blocks = {}

        def block(az, ay, ax):
            return np.ascontiguousarray(host[az * 32:az * 32 + 32, ay * 32:ay * 32 + 32, ax * 32:ax * 32 + 32])

        for mode, nthreads in (("append_atom", threads), ("append_atom_async", 1), ("append_atom_async", threads)):
            path = os.path.join(td, f"{mode}_{nthreads}.vca")
            w = vc.Writer(path, dims, 10.0)
            assert w.set_base_q(0, q0) == 0
            bad = []
            fn = w.append_atom if mode == "append_atom" else w.append_atom_async
            # each synchronous call waits for one coder chain: time it on the first sync_atoms atoms
            todo = atoms[:sync_atoms] if mode == "append_atom" else atoms

            def worker(k):
                for az, ay, ax in todo[k::nthreads]:
                    if fn(0, az, ay, ax, block(az, ay, ax)) != 0:
                        bad.append((az, ay, ax))
            th = [threading.Thread(target=worker, args=(k,)) for k in range(nthreads)]
            t0 = time.perf_counter()
            for t in th:
                t.start()
            for t in th:
                t.join()
            if mode != "append_atom":
                fs, nf = w.flush()
                if fs:
                    bad.append(("flush", fs, nf))
            w.close()
            t1 = time.perf_counter() - t0
            row = {"atoms": len(todo), "s": t1, "GBps": len(todo) * 32768 / t1 / 1e9, "failed": len(bad),
                   "file_bytes": os.path.getsize(path)}
            if len(todo) == len(atoms):
                row["lod0_matches_reference"] = check(path)
            res[f"{mode}_{nthreads}threads"] = row
        del blocks
    # CPU leg: the oracle's per-atom encode on a sample of atoms
    O = oraclelib.lib()
    rng = np.random.default_rng(0xC0DE)
    ids = np.sort(rng.choice((nx // 32) * (ny // 32) * (nz // 32), cpu_sample, replace=False)).astype(np.uint32)
    lens = np.zeros(cpu_sample, np.uint32)
    t0 = time.perf_counter()
    O.orc_encode_sizes_mt(host.ctypes.data, oraclelib.Dims(nx, ny, nz), ctypes.c_float(q0), ids.ctypes.data,
                          cpu_sample, lens.ctypes.data, threads)
    t_cpu = time.perf_counter() - t0
    res["cpu_port"] = {"GBps": cpu_sample * 32768 / t_cpu / 1e9, "threads": threads, "kind": "port",
                       "sample": f"{cpu_sample} atoms of the volume, sizes only (no file)"}
    return res


def config3_dct(n=1024, reps=3, sample_atoms=256):
    """Whole-atom integer DCT of the 1024^3 volume, x = vox - dc per atom as the
    codec centres, forward and inverse, in both forms: butterfly (CUDA cores)
    and IMMA (int8 tensor cores, hi/lo pieces). Every coefficient, dc and voxel
    of the two forms is compared; the CPU leg times the C restatement of the
    reference transform on a bounded sample of atoms and checks the device
    outputs of those atoms."""
    import numpy as np
    import vc_gb300 as vc
    dims = (n, n, n)
    centre = vc.DCT_ATOM_DC
    vol = vc.synth_device(n, n, n, vc.config_seed(3))
    coef = [vc.DeviceBuffer(n ** 3 * 4) for _ in range(2)]
    rec = [vc.DeviceBuffer(n ** 3) for _ in range(2)]
    dcs = [vc.DeviceBuffer(n ** 3 // 32768) for _ in range(2)]
    res = {}
    for form, name in ((vc.DCT_BUTTERFLY, "butterfly"), (vc.DCT_IMMA, "imma")):
        fwd, inv = [], []
        for r in range(reps + 1):
            s, redone = vc.dct_forward(vol, dims, centre, form, coef[form], dcs[form])
            assert s == 0 and redone == 0, vc.last_error()
            if r or not reps:
                fwd.append(vc.last_call_ms())
        for r in range(reps + 1):
            s, redone = vc.dct_inverse(coef[form], dims, centre, form, rec[form], dcs[form])
            assert s == 0, vc.last_error()
            if r or not reps:
                inv.append(vc.last_call_ms())
        f, i = min(fwd), min(inv)
        res[name] = {"forward_ms": f, "inverse_ms": i, "inverse_atoms_redone": redone,
                     "forward_voxel_GBps": n ** 3 / (f / 1e3) / 1e9,
                     "forward_hbm_GBps": 5 * n ** 3 / (f / 1e3) / 1e9,
                     "inverse_voxel_GBps": n ** 3 / (i / 1e3) / 1e9,
                     "inverse_hbm_GBps": 5 * n ** 3 / (i / 1e3) / 1e9}
    forms_equal = (_equal_device(vc, coef[0], coef[1], n ** 3 * 4) and _equal_device(vc, rec[0], rec[1], n ** 3)
                   and _equal_device(vc, dcs[0], dcs[1], n ** 3 // 32768))
    dc_host = dcs[1].download(n ** 3 // 32768)
    # CPU leg: the C restatement of the reference transform on a bounded sample of atoms
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oraclelib
    O = oraclelib.lib()
    rng = np.random.default_rng(0xD7C3)
    na = n // 32
    picks = rng.choice(na ** 3, min(sample_atoms, na ** 3), replace=False)
    host_vol = np.empty((32, 32, 32), np.uint8)
    ok = True
    t_cpu = 0.0
    L = vc.lib()
    for a in picks:
        a = int(a)
        ax, ay, az = a % na, (a // na) % na, a // (na * na)
        for z in range(32):
            for y in range(32):
                L.vcg_copy(host_vol[z, y].ctypes.data,
                           ctypes.c_void_p(vol.ptr + ((az * 32 + z) * n + ay * 32 + y) * n + ax * 32), 32)
        c_ref = np.empty(32768, np.int32)
        v_ref = np.empty(32768, np.uint8)
        t0 = time.perf_counter()
        dc = (int(host_vol.sum(dtype=np.int64)) + 16384) // 32768
        O.orc_fdct(host_vol.ctypes.data, dc, c_ref.ctypes.data)
        O.orc_idct(c_ref.ctypes.data, dc, v_ref.ctypes.data)
        t_cpu += time.perf_counter() - t0
        ok = ok and dc == int(dc_host[a])
        c_dev = np.empty(32768, np.int32)
        L.vcg_copy(c_dev.ctypes.data, ctypes.c_void_p(coef[1].ptr + a * 32768 * 4), 32768 * 4)
        v_dev = np.empty((32, 32, 32), np.uint8)
        for z in range(32):
            for y in range(32):
                L.vcg_copy(v_dev[z, y].ctypes.data,
                           ctypes.c_void_p(rec[1].ptr + ((az * 32 + z) * n + ay * 32 + y) * n + ax * 32), 32)
        ok = ok and bool(np.array_equal(c_dev, c_ref)) and bool(np.array_equal(v_dev.ravel(), v_ref))
    for b in coef + rec + dcs + [vol]:
        b.free()
    return {"workload": f"{n}^3 u8 synthetic volume (seed 0x5EED0003), {na ** 3} atoms, x = vox - dc per atom, "
                        "forward + inverse 3-D DCT-32",
            **res, "imma_vs_butterfly_forward_speedup": res["butterfly"]["forward_ms"] / res["imma"]["forward_ms"],
            "imma_vs_butterfly_inverse_speedup": res["butterfly"]["inverse_ms"] / res["imma"]["inverse_ms"],
            "forms_identical_all_outputs": forms_equal,
            "cpu_reference": {"atoms": sample_atoms, "threads": 1, "kind": "port",
                              "voxel_MBps_forward_plus_inverse": sample_atoms * 32768 / t_cpu / 1e6,
                              "bit_exact_sample": ok}}


def served_mix(a, rng, n):
    """Request mix of the served-decode workload: 70% single 32^3 atoms at LOD0,
    25% boxes with edges U[64,128] at LOD 0-1, 5% 512^3 boxes at LOD2."""
    reqs = []
    for _ in range(n):
        u = rng.random()
        if u < 0.70:
            d = a.lod_dims(0)[1]
            o = [32 * int(rng.integers(0, (d[k] + 31) // 32)) for k in range(3)]
            e = [min(32, d[k] - o[k]) for k in range(3)]
            lod = 0
        elif u < 0.95:
            lod = int(rng.integers(0, 2))
            d = a.lod_dims(lod)[1]
            e = [int(min(rng.integers(64, 129), d[k])) for k in range(3)]
            o = [int(rng.integers(0, d[k] - e[k] + 1)) for k in range(3)]
        else:
            lod = 2
            d = a.lod_dims(2)[1]
            e = [min(512, d[k]) for k in range(3)]
            o = [int(rng.integers(0, d[k] - e[k] + 1)) for k in range(3)]
        reqs.append((lod, (o[0], o[1], o[2], o[0] + e[0], o[1] + e[1], o[2] + e[2])))
    return reqs


def _box_bytes(b):
    return (b[3] - b[0]) * (b[4] - b[1]) * (b[5] - b[2])


def _pace(t0, arrival):
    while True:
        dt = t0 + arrival - time.perf_counter()
        if dt <= 0:
            return
        time.sleep(dt if dt > 2e-3 else 0)


def _serve_stream(a, reqs, arrivals, outs, server_cfg):
    """One Poisson stream through the decode server. Returns per-request
    latencies (µs, submit to completion) and the wall time first arrival -> last
    completion."""
    import numpy as np
    srv = a.server(**server_cfg)
    tix = [None] * len(reqs)
    lat = np.zeros(len(reqs))
    status = np.zeros(len(reqs), np.int32)
    ready = threading.Semaphore(0)

    def waiter():
        for i in range(len(reqs)):
            ready.acquire()
            status[i], lat[i] = srv.wait(tix[i])
    th = threading.Thread(target=waiter)
    th.start()
    t0 = time.perf_counter()
    for i, (lod, box) in enumerate(reqs):
        _pace(t0, arrivals[i])
        tix[i] = srv.submit(lod, box, outs[i])
        ready.release()
    th.join()
    wall = time.perf_counter() - t0
    batches, done = srv.stats()
    srv.close()
    assert not status.any(), f"server statuses {np.unique(status)}"
    return lat, wall, done / max(1, batches)


def _plain_stream(a, reqs, arrivals, outs, workers):
    """The same stream through the plain per-request path: `workers` threads take
    requests in arrival order and call vc_decode_region one at a time."""
    import numpy as np
    lat = np.zeros(len(reqs))
    status = np.zeros(len(reqs), np.int32)
    nxt = [0]
    mu = threading.Lock()
    t0 = time.perf_counter()

    def run():
        while True:
            with mu:
                i = nxt[0]
                nxt[0] += 1
            if i >= len(reqs):
                return
            _pace(t0, arrivals[i])
            status[i] = a.decode_region(reqs[i][0], reqs[i][1], outs[i])[0]
            lat[i] = (time.perf_counter() - t0 - arrivals[i]) * 1e6
    th = [threading.Thread(target=run) for _ in range(workers)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    wall = time.perf_counter() - t0
    assert not status.any(), f"plain statuses {np.unique(status)}"
    return lat, wall


def config5_served(rates=(100, 300, 1000, 3000), seconds=1.5, max_requests=3000, verify_n=400):
    """Served decode: 2048^3 volume at target_ratio 20 resident in HBM; Poisson
    request streams at swept rates through the continuous-batching server
    (vcg_server_*) and through the plain per-request path (vc_decode_region on
    as many host threads as the server has workers). Outputs are host memory;
    large-box outputs rotate through a pool in the timed streams, and a separate
    stream of verify_n requests with distinct outputs is checked byte for byte
    against the CPU's decode of each request (the CPU baseline's sample)."""
    import numpy as np
    import vc_gb300 as vc
    n = 2048
    dv = vc.synth_device(n, n, n, vc.config_seed(5))
    s, data, q0 = vc.encode_device(dv, (n, n, n), 20.0)
    assert s == 0, vc.last_error()
    dv.free()
    a = vc.Archive(data)
    assert a.make_resident() == 0
    cfg = {"device_budget": 2 << 30, "max_batch": 1024, "workers": int(os.environ.get("VC_BENCH_SERVER_WORKERS", "3"))}
    rng = np.random.default_rng(0x5E5E)
    warm = served_mix(a, rng, 64)   # first batches tune the launch shape and build graphs
    wo = [np.empty(_box_bytes(b), np.uint8) for _, b in warm]
    _serve_stream(a, warm, np.zeros(len(warm)), wo, cfg)
    big_pool = [np.empty(512 ** 3, np.uint8) for _ in range(8)]
    sweep = []
    for rate in rates:
        m = int(min(max_requests, max(1500, rate * seconds)))   # at least ~75 large requests per rate
        reqs = served_mix(a, rng, m)
        arrivals = np.cumsum(rng.exponential(1.0 / rate, m))
        outs, k = [], 0
        for _, b in reqs:
            nb = _box_bytes(b)
            if nb == 512 ** 3:
                outs.append(big_pool[k % len(big_pool)])
                k += 1
            else:
                outs.append(np.empty(nb, np.uint8))
        total = sum(_box_bytes(b) for _, b in reqs)
        row = {"offered_rps": rate, "requests": m, "out_bytes": total}
        for name, fn in (("server", lambda: _serve_stream(a, reqs, arrivals, outs, cfg)),
                         ("plain", lambda: _plain_stream(a, reqs, arrivals, outs, cfg["workers"]))):
            r = fn()
            lat, wall = r[0], r[1]
            lat_a = np.asarray(lat)
            big = np.array([_box_bytes(b) >= (32 << 20) for _, b in reqs])
            row[name] = {"p50_us": float(np.percentile(lat, 50)), "p99_us": float(np.percentile(lat, 99)),
                         "GBps": total / wall / 1e9, "achieved_rps": m / wall,
                         "small": {"p50_us": float(np.percentile(lat_a[~big], 50)),
                                   "p99_us": float(np.percentile(lat_a[~big], 99))} if (~big).any() else None,
                         "large_512": {"p50_us": float(np.percentile(lat_a[big], 50)),
                                       "p99_us": float(np.percentile(lat_a[big], 99))} if big.any() else None}
            if name == "server":
                row[name]["mean_batch"] = r[2]
        sweep.append(row)
    # bit-exactness: distinct outputs, highest rate, every request checked
    reqs = served_mix(a, rng, verify_n)
    arrivals = np.cumsum(rng.exponential(1.0 / rates[-1], verify_n))
    outs = [np.empty(_box_bytes(b), np.uint8) for _, b in reqs]
    _serve_stream(a, reqs, arrivals, outs, cfg)
    # the reference's decode of the same archive: the golden requests served
    import hashlib
    g = golden_named("cfg5_2048_t20")
    arc_ok = None if g is None else g["sha256"] == hashlib.sha256(data).hexdigest()
    ref_ok, ref_n = (None if g is None else False), 0
    if arc_ok:
        greqs = [(r["lod"], tuple(r["box"])) for r in g["requests"]]
        gouts = [np.empty(_box_bytes(b), np.uint8) for _, b in greqs]
        _serve_stream(a, greqs, np.zeros(len(greqs)), gouts, cfg)
        ref_ok = all(hashlib.sha256(o.tobytes()).hexdigest() == r["sha256"] for o, r in zip(gouts, g["requests"]))
        ref_n = len(greqs)
        del gouts
    a.close()
    # every served output against the CPU's decode of the same request (the
    # CPU baseline's all-threads pass); one thread on the first requests
    ok = [True]

    def same(i, out):
        ok[0] = ok[0] and bool(np.array_equal(outs[i], out))
    cpu = None
    if os.environ.get("VC_BENCH_NO_CPU") != "1":
        cpu = cpu_regions(data, reqs, one_n=60, all_n=verify_n, budget_s=10.0, check=same)
    ok = ok[0] if cpu else None
    return {"workload": "2048^3 at target_ratio 20 resident in HBM; Poisson arrivals; 70% 32^3 atoms LOD0, "
                        "25% boxes U[64,128]^3 LOD0-1, 5% 512^3 LOD2; host outputs",
            "q0": q0, "archive_bytes": len(data), "server": cfg, "plain_threads": cfg["workers"],
            "sweep": sweep, "bit_exact_all_outputs_vs_cpu": ok, "verified_requests": verify_n,
            "bit_exact_vs_reference": {"archive": arc_ok, "requests": ref_ok, "requests_checked": ref_n},
            "cpu_baseline": cpu}


# ---------------------------------------------------------------- arms
def reference_arm(args, dist):
    if dist.rank != 0:
        return
    threads = os.cpu_count() or 1
    data, q0 = cpu_decode_setup(args.size, args.target, threads)
    kind, run = cpu_decoder(data, threads)
    for _ in range(args.warmup):
        run()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run()
    dt = time.perf_counter() - t0
    nbytes = args.size ** 3
    gbps = args.steps * nbytes / dt / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": gbps, "unit": "GB/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "i32",
            "data": "synthetic",
            "config": {"workload": f"LOD0 decode, {args.size}^3 u8 synthetic scroll volume, target_ratio "
                                   f"{args.target:g}", "q0": q0, "archive_bytes": len(data)},
            "cpu_baseline": dict({"value": gbps, "unit": "GB/s", "cores": threads, "kind": kind,
                                  "sample": f"full LOD0 decode ({nbytes} voxels) per step, parallel-for over atoms"},
                                 **host_info()),
            "e2e": {"value": gbps, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(_round(line), separators=(",", ":")), flush=True)


def gb300_arm(args, dist):
    import numpy as np
    import vc_gb300 as vc
    if not os.path.exists(vc.LIB_PATH):
        vc.build()
    n = args.size
    nbytes = n ** 3
    dims = (n, n, n)
    s, nsm, cc = vc.device_info()
    assert s == 0, vc.last_error()
    g = golden_case(n, args.target)

    # workload: synthetic volume on the device, encoded by this library
    dvol = vc.synth_device(n, n, n, vc.config_seed(CONFIG_ID))
    s, data, q0 = vc.encode_device(dvol, dims, args.target)
    assert s == 0, vc.last_error()
    enc_full_ms = vc.last_call_ms()
    qs, q = [], np.float32(q0)
    for _ in range(8):
        qs.append(float(max(q, np.float32(0.05))))
        q = np.float32(q * np.float32(0.6))
    enc_ms = []
    for _ in range(2):
        s, data_q = vc.encode_q(dvol, args.target, qs, on_device=dims)
        assert s == 0 and data_q == data
        enc_ms.append(vc.last_call_ms())
    bit_exact_archive = (g["sha256"] == __import__("hashlib").sha256(data).hexdigest()) if g else None

    arc = vc.Archive(data)
    assert arc.make_resident() == 0
    out = vc.DeviceBuffer(nbytes)
    flush = vc.DeviceBuffer(512 << 20)
    for _ in range(args.warmup):
        assert arc.decode_lod_device(0, out) == 0
    lod0_ok = None
    if g:
        import hashlib
        lod0_ok = hashlib.sha256(out.download(nbytes).tobytes()).hexdigest() == g["lod_sha256"][0]

    vc.profile_enable(True)
    vc.profile_read(reset=True)
    dist.barrier()
    vc.sync()
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    ms = []
    for k in range(args.steps):
        vc.lib().vcg_memset(flush.ptr, k & 0xFF, flush.nbytes)   # L2 flush, not timed
        assert arc.decode_lod_device(0, out) == 0
        ms.append(vc.last_call_ms())
    vc.sync()
    clk = clocks.stop()
    dist.barrier()
    stats = vc.profile_read(reset=True)
    vc.profile_enable(False)
    total_ms = dist.max(sum(ms))
    value = dist.sum(args.steps * nbytes) / (total_ms / 1e3) / 1e9

    # e2e through the drop-in ABI with pinned host buffers
    L = vc.lib()
    hp = L.vcg_alloc_host(len(data))
    ctypes.memmove(hp, data, len(data))
    ho = L.vcg_alloc_host(nbytes)
    d = vc.Dims()
    e2e_t = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        h = L.vc_open(hp, len(data))
        st = L.vc_decode_lod(h, 0, ho, ctypes.byref(d))
        L.vc_close(h)
        t1 = time.perf_counter()
        assert st == 0
        if k >= args.warmup:
            e2e_t.append(t1 - t0)
    e2e_s = dist.max(sum(e2e_t))
    e2e = dist.sum(args.steps * nbytes) / e2e_s / 1e9
    # the same calls with the output in pageable memory (a malloc'd buffer, as a
    # drop-in caller of the reference API passes it; already touched)
    pg = np.full(nbytes, 0x5A, np.uint8)
    pg_t = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        h = L.vc_open(hp, len(data))
        st = L.vc_decode_lod(h, 0, pg.ctypes.data, ctypes.byref(d))
        L.vc_close(h)
        t1 = time.perf_counter()
        assert st == 0
        if k >= args.warmup:
            pg_t.append(t1 - t0)
    e2e_pg = dist.sum(args.steps * nbytes) / dist.max(sum(pg_t)) / 1e9
    del pg
    L.vcg_free_host(hp)
    L.vcg_free_host(ho)

    # per-request region latency (plain path, host output)
    rng = np.random.default_rng(0xB0C5)
    lat, region_reqs = [], []
    for _ in range(args.regions):
        lod = int(rng.integers(0, 4))
        dd = arc.lod_dims(lod)[1]
        e = [int(min(rng.integers(32, 257), dd[k])) for k in range(3)]
        o = [int(rng.integers(0, dd[k] - e[k] + 1)) for k in range(3)]
        box = (o[0], o[1], o[2], o[0] + e[0], o[1] + e[1], o[2] + e[2])
        t0 = time.perf_counter()
        st, _ = arc.decode_region(lod, box)
        lat.append((time.perf_counter() - t0) * 1e6)
        assert st == 0
        region_reqs.append((lod, box))
    lat.sort()
    region_cpu = None
    if dist.rank == 0 and os.environ.get("VC_BENCH_NO_CPU") != "1":
        region_cpu = cpu_regions(data, region_reqs, one_n=30, all_n=len(region_reqs))

    # roofline of the dominant stage
    peak, peak_kind = measured_peak()
    dom = max((k for k in stats if k in ("idct", "rc_decode", "decode_fused")), key=lambda k: stats[k]["ms"])
    st_ = stats[dom]
    # per step of the stage (one decode call): the range-decode stage is the
    # per-lane decoder's launch after three small length-sort launches
    per_launch_bytes = (st_["bytes_read"] + st_["bytes_written"]) / args.steps
    per_launch_ms = st_["ms"] / args.steps
    achieved = per_launch_bytes / (per_launch_ms / 1e3) / 1e9
    launches = int(sum(v["launches"] for v in stats.values()))

    cpu = None
    if dist.rank == 0 and os.environ.get("VC_BENCH_NO_CPU") != "1":
        threads = os.cpu_count() or 1
        kind, run = cpu_decoder(data, threads)
        t0 = time.perf_counter()
        ref_out = run()
        dt = time.perf_counter() - t0
        cpu = {"value": nbytes / dt / 1e9, "unit": "GB/s", "cores": threads, "kind": kind,
               "sample": f"one full LOD0 decode ({nbytes} voxels) of the same archive, parallel-for over atoms"}
        v1, k1, s1 = cpu_one_thread(data)
        cpu["one_thread"] = {"value": v1, "unit": "GB/s", "kind": k1, "sample": s1}
        cpu.update(host_info())
        if lod0_ok is None:
            lod0_ok = bool(np.array_equal(out.download(nbytes), ref_out.ravel()))

    sweep = ds = atom = None
    if dist.rank == 0 and not args.no_sweep:
        sweep = config2_sweep(dvol, dims, peak)
    if dist.rank == 0 and not args.no_atom:
        atom = atom_latency(dvol, dims)
    if dist.rank == 0 and not args.no_ds:
        ds = downscale_bench(dvol, dims, peak)
    writer = None
    if dist.rank == 0 and not args.no_writer:
        writer = writer_bench(dvol, dims, q0, g)
    # the other workloads (rank 0): release the headline buffers first
    batched = dct = served = None
    if dist.rank == 0 and not (args.no_batched and args.no_dct and args.no_served):
        arc.close()
        out.free()
        flush.free()
        dvol.free()
        if not args.no_batched:
            batched = config4_batched()
        if not args.no_dct:
            dct = config3_dct(n=args.dct_size, reps=args.dct_reps)
        if not args.no_served:
            served = config5_served()
    if dist.rank != 0:
        return
    roof = {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": dram_traffic(dom, st_["units"] / args.steps),
            "peak_source": peak_kind}
    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": dist.world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "i32", "data": "synthetic",
        "config": {"workload": f"LOD0 decode, {n}^3 u8 synthetic scroll volume (seed 0x5EED0002), "
                               f"target_ratio {args.target:g}, archive resident in HBM",
                   "l2": "flushed between timed steps (512 MiB device write)", "parallelism": f"replicas{dist.world}"},
        "e2e": {"value": e2e, "unit": "GB/s", "h2d_bytes_per_step": len(data), "d2h_bytes_per_step": nbytes},
        "gpu_launches": launches,
        "roofline": roof,
        "clocks": {k: clk.get(k) for k in ("sm_mhz", "sm_max_mhz", "reasons")},
        "bit_exact": {"archive_vs_reference": bit_exact_archive, "lod0_vs_reference": lod0_ok},
        "region_p50_us": lat[len(lat) // 2] if lat else None,
        "region_p99_us": lat[min(len(lat) - 1, int(len(lat) * 0.99))] if lat else None,
    }
    if cpu:
        line["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
    # everything else goes to the side file and to one earlier stdout line
    detail = dict(line)
    detail["config"] = dict(line["config"], volume=list(dims), target_ratio=args.target, q0=q0,
                            archive_bytes=len(data))
    detail["e2e"] = dict(line["e2e"], step_ms=[round(t * 1e3, 3) for t in e2e_t])
    detail["e2e_pageable"] = {"value": e2e_pg, "unit": "GB/s", "step_ms": [round(t * 1e3, 3) for t in pg_t],
                              "note": "same calls, output in pageable memory (copied out through pinned bounce chunks)"}
    detail["roofline"] = dict(roof, algorithmic_bytes_per_launch=per_launch_bytes, ms_per_launch=per_launch_ms,
                              limiter=LIMITER.get(dom))
    detail["clocks"] = clk
    detail["stages"] = {k: {"ms_per_step": v["ms"] / args.steps, "GBps_algorithmic":
                            (v["bytes_read"] + v["bytes_written"]) / max(1e-9, v["ms"] / 1e3) / 1e9}
                        for k, v in stats.items()}
    detail["encode_GBps"] = nbytes / (statistics.median(enc_ms) / 1e3) / 1e9
    if region_cpu:
        detail["region_latency_cpu"] = region_cpu
    detail["encode_with_rate_control_GBps"] = nbytes / (enc_full_ms / 1e3) / 1e9
    if cpu:
        detail["cpu_baseline"] = cpu
    for key, val in (("batched_regions", batched), ("served_regions", served), ("dct_forms", dct),
                     ("config2_sweep", sweep), ("atom_latency", atom), ("exporter_downscale", ds),
                     ("writer_append", writer)):
        if val:
            detail[key] = val
    emit(line, detail, args.detail)


def _round(v):
    if isinstance(v, float):
        return float(f"{v:.5g}")
    if isinstance(v, dict):
        return {k: _round(x) for k, x in v.items()}
    if isinstance(v, list):
        return [_round(x) for x in v]
    return v


def emit(line, detail, path):
    """Writes the full record to `path` and as one stdout line tagged
    "detail", then prints the headline as the LAST stdout line, compact (floats
    to 5 significant digits), so that a reader that keeps only the tail of the
    output still gets the whole headline object."""
    if path:
        try:
            os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
            with open(path, "w") as f:
                json.dump(detail, f, indent=1)
        except OSError as e:
            print(f"bench: cannot write {path}: {e}", file=sys.stderr)
    print(json.dumps({"detail": detail}), flush=True)
    sys.stderr.flush()
    out = json.dumps(_round(line), separators=(",", ":"))
    print(out, flush=True)


def main():
    args = args_parse()
    dist = Dist()
    if args.impl == "reference":
        reference_arm(args, dist)
    else:
        gb300_arm(args, dist)


if __name__ == "__main__":
    main()
