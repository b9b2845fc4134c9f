"""sc_kick_host (particles and outputs in host memory, chunked copies
overlapping the deposit and the gather) against sc_kick on device arrays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return np.abs(a - b).max() / np.abs(b).max()


def bunch(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((3, n)).clip(-4.5, 4.5) * np.array([[1e-3], [1e-3], [2e-4]])
    return v[0], v[1], np.abs(v[2]) + 0.05e-3


@pytest.mark.parametrize("prec,mode", [("mixed", "vector"), ("mixed", "atomic"), ("mixed", "sorted"),
                                       ("fp64", "atomic"), ("df32", "atomic"), ("plain64", "atomic")])
@pytest.mark.parametrize("cath", [False, True])
def test_kick_host_matches_device_kick(sc, cuda, prec, mode, cath):
    """df32: an FP64 mesh in double-FP32 mode."""
    import torch

    n = 300_001  # not a multiple of the chunk count
    x, y, z = bunch(n, 5)
    q = np.full(n, 1e-9 / n)
    m = sc.Mesh3D((24, 20, 40), x, y, z, precision="fp64" if prec == "df32" else prec, gamma=3.0)
    if prec == "df32":
        m.set_fp64_arithmetic("df32")
    if prec != "plain64":
        m.set_kick_mode(mode)
    hx, hy, hz, hq = (torch.from_numpy(a).pin_memory() for a in (x, y, z, q))
    eh = sc.kick_host(m, hx, hy, hz, hq, at_cathode=cath)
    ed = sc.kick(m, x, y, z, q, at_cathode=cath)
    # FP64: the atomic deposit's summation order differs between the two kicks
    tol = 1e-5 if prec == "mixed" else 1e-10
    for a, b in zip(eh, ed):
        assert not a.is_cuda
        assert rel(a.numpy(), b) < tol


def test_kick_host_float32_pageable_and_repeat(sc, cuda):
    n = 70_000
    x, y, z = (a.astype(np.float32) for a in bunch(n, 6))
    q = np.full(n, 1e-9 / n, dtype=np.float32)
    m = sc.Mesh3D((16, 16, 16), x, y, z, precision="mixed")
    ref = sc.kick(m, x, y, z, q)
    for _ in range(3):  # pageable numpy inputs, repeated calls reuse the staging
        e = sc.kick_host(m, x, y, z, q)
        for a, b in zip(e, ref):
            assert a.dtype == __import__("torch").float32
            assert rel(a.numpy(), b) < 1e-5
    with pytest.raises(sc.SpaceChargeError):
        sc.kick_host(m, x, y[:-1], z, q)
