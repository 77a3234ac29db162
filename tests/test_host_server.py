"""The decode server (volume-compressor_gb300/csrc/vc_server.c) built for the
host against stand-in decode calls (tests/host_server.c), no GPU: mixed
request streams with 1, 3 and 8 workers and tight or loose device budgets,
whole batched calls that fail, a small request arriving behind queued large
ones, requests that each exceed the budget, and a destroy with requests still
queued. Each scenario checks that every request is decoded once into its own
output with its own status, that batches stay within max_batch, one size class
and the device budget, and the ticket rules (recycled slots, a second wait
refused). Reference behaviour served: vc_decode_region per request
(src/vc/vc.c:1535-1555)."""
import os
import subprocess

import pytest

from conftest import ROOT


def test_server_scenarios(tmp_path):
    exe = str(tmp_path / "host_server")
    srcs = [os.path.join(ROOT, "tests", "host_server.c"),
            os.path.join(ROOT, "volume-compressor_gb300", "csrc", "vc_server.c")]
    r = subprocess.run(["gcc", "-O2", "-std=gnu11", "-I", os.path.join(ROOT, "include"), *srcs, "-lpthread",
                        "-o", exe], capture_output=True, text=True)
    if r.returncode:
        pytest.fail(r.stderr[-2000:])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    lines = r.stdout.strip().splitlines()
    assert r.returncode == 0, r.stdout + r.stderr
    assert len(lines) == 7 and all(line.endswith(" ok") for line in lines), r.stdout
