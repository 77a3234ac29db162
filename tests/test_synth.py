"""The seeded synthetic workload generator: deterministic, slab-independent,
and identical between the host library and the CUDA generator."""
import hashlib

import numpy as np
import pytest


def test_host_generator_is_deterministic_and_slab_independent(vc):
    a = vc.synth(80, 70, 90, 123, threads=4)
    b = vc.synth(80, 70, 90, 123, threads=1)
    assert (a == b).all()
    s = vc.synth(80, 70, 90, 123, z0=31, z1=77)
    assert (s == a[31:77]).all()
    c = vc.synth(80, 70, 90, 124)
    assert not (a == c).all()


def test_host_generator_statistics(vc):
    v = vc.synth(128, 128, 120, vc.config_seed(1))
    assert 10 < v.mean() < 120
    assert (v >= 230).sum() > 0                 # inclusions
    assert ((v > 100) & (v < 200)).mean() > 0.1   # sheets


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(64, 64, 64), (97, 131, 65), (256, 256, 256), (33, 1, 700)])
def test_device_generator_matches_host(vc, gpu, dims):
    nx, ny, nz = dims
    h = vc.synth(nx, ny, nz, 77)
    d = vc.synth_device(nx, ny, nz, 77)
    assert (d.download(nx * ny * nz) == h.ravel()).all()
