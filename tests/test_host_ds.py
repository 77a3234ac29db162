"""The device's 2x2x2 cell values of the exporter downscale (ds_cell.cuh:
DS_BOX, and DS_CBOX with the push toward the cell's voxel of largest deviation
as one fused multiply-add or as a multiply and an add) built for the host
(tests/host_ds.cpp) and checked against the oracle's cell rule
(oracle/vc_oracle.c orc_ds_cell, pinned to the reference's tools/downscale.h
build): random cells, cells with tied deviations, flat, zero and extreme cells,
cells of the synthetic volume, and the cells where the fused and the separate
push round to different bytes, at several alphas (the separating one among
them). No GPU needed."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from test_downscale import SEPARATING, separating_cells


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    exe = str(tmp_path_factory.mktemp("host_ds") / "host_ds")
    src = os.path.join(ROOT, "tests", "host_ds.cpp")
    inc = os.path.join(ROOT, "volume-compressor_gb300", "csrc")
    r = subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-w", "-I", inc, src, "-o", exe],
                       capture_output=True, text=True)
    if r.returncode:
        pytest.fail(r.stderr[-2000:])
    return exe


def oracle_cells(oracle, cells, method, alpha, fused):
    L = oracle.lib()
    L.orc_ds_set_fused(1 if fused else 0)
    try:
        out = np.empty(len(cells), np.uint8)
        for i, c in enumerate(cells):
            out[i] = L.orc_ds_cell(c.ctypes.data, method, np.float32(alpha))
        return out
    finally:
        L.orc_ds_set_fused(1)


def cell_set(vc, oracle):
    rng = np.random.default_rng(0xD5C)
    cells = [rng.integers(0, 256, 8).astype(np.uint8) for _ in range(6000)]
    for _ in range(3000):   # small deviations around a level
        base = int(rng.integers(0, 256))
        cells.append(np.clip(base + rng.integers(-3, 4, 8), 0, 255).astype(np.uint8))
    for _ in range(1000):   # tied largest deviations
        c = np.full(8, int(rng.integers(20, 236)), np.int64)
        i, j = rng.choice(8, 2, replace=False)
        d = int(rng.integers(1, 20))
        c[i] += d
        c[j] -= d
        cells.append(c.astype(np.uint8))
    cells += [np.zeros(8, np.uint8), np.full(8, 255, np.uint8), np.array([255, 0] * 4, np.uint8),
              np.array([0] * 7 + [255], np.uint8), np.array([1] + [0] * 7, np.uint8)]
    vol = vc.synth(64, 64, 64, vc.config_seed(3))
    for z in range(0, 64, 16):
        for y in range(0, 64, 8):
            for x in range(0, 64, 2):
                cells.append(np.ascontiguousarray(vol[z:z + 2, y:y + 2, x:x + 2]).ravel())
    # cells where the two push forms round to different bytes (at the separating alpha)
    sep = [np.asarray(c, np.uint8) for c, _, _ in separating_cells(SEPARATING[0])]
    cells += sep
    return [np.ascontiguousarray(c, np.uint8) for c in cells], len(sep)


def test_cells_match_oracle(vc, oracle, harness, tmp_path):
    cells, nsep = cell_set(vc, oracle)
    assert nsep > 0
    fi, fo = str(tmp_path / "cells.bin"), str(tmp_path / "out.bin")
    np.concatenate(cells).tofile(fi)
    for method, alphas in ((0, (0.5,)), (1, (0.5, 0.3, SEPARATING[0], 0.7, 1.0, 0.0, 0.123))):
        for alpha in alphas:
            for fused in ((True,) if method == 0 else (True, False)):
                r = subprocess.run([harness, fi, fo, str(method), repr(float(np.float32(alpha))),
                                    "1" if fused else "0"], capture_output=True, text=True, timeout=300)
                assert r.returncode == 0, r.stderr
                got = np.fromfile(fo, np.uint8)
                want = oracle_cells(oracle, cells, method, alpha, fused)
                bad = np.nonzero(got != want)[0]
                assert len(bad) == 0, (method, alpha, fused, len(bad), cells[bad[0]])
