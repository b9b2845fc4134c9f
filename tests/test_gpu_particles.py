"""Beside the kick: the bunch's magnetic field at the particles and the
particle-layout adapters (array-of-structs records, FP32 positions relative
to an FP64 point)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def bunch(n, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((3, n)).clip(-4.5, 4.5) * 1e-3


@pytest.mark.parametrize("gamma", [1.0, 1.01, 10.0])
def test_magnetic_field_is_beta_z_cross_e(sc, cuda, gamma):
    x, y, z = bunch(20_000, 1)
    q = np.full(x.size, 1e-9 / x.size)
    m = sc.Mesh3D((16, 16, 16), x, y, z, precision="fp64", gamma=gamma)
    ex, ey, ez = sc.kick(m, x, y, z, q)
    bx, by = sc.magnetic_field(m, ex, ey)
    beta = np.sqrt(1 - 1 / gamma**2)
    assert np.allclose(bx, -beta * ey / O.CLIGHT, rtol=1e-14, atol=0)
    assert np.allclose(by, beta * ex / O.CLIGHT, rtol=1e-14, atol=0)


@pytest.mark.parametrize("dt", ["float64", "float32"])
def test_aos_records_round_trip_through_the_kick(sc, cuda, dt):
    import torch

    n = 50_000
    x, y, z = bunch(n, 2)
    q = np.full(n, 1e-9 / n)
    tdt = getattr(torch, dt)
    # records (x, px, y, py, z, pz, q, Ex, Ey, Ez): positions, charge and outputs interleaved
    rec = torch.zeros((n, 10), dtype=tdt, device="cuda")
    rec[:, 0], rec[:, 2], rec[:, 4], rec[:, 6] = (torch.as_tensor(a, dtype=tdt) for a in (x, y, z, q))
    rx, ry, rz, rq = sc.aos_to_soa(rec, offsets=(0, 2, 4, 6))
    assert torch.equal(rx, rec[:, 0]) and torch.equal(rq, rec[:, 6])
    m = sc.Mesh3D((16, 16, 24), x, y, z, precision="mixed")
    e = sc.kick(m, rx, ry, rz, rq)
    sc.soa_to_aos(*e, rec, offsets=(7, 8, 9))
    for c in range(3):
        assert torch.equal(rec[:, 7 + c], e[c])
    with pytest.raises(sc.SpaceChargeError):
        sc.aos_to_soa(rec, offsets=(0, 2, 4, 10))


def test_relative_positions_far_from_the_origin(sc, cuda):
    """FP32 offsets from an FP64 centroid 1 km away give the same kick as the
    FP64 absolute positions."""
    n = 40_000
    r = bunch(n, 3).astype(np.float32)
    ref = (1000.0, -250.0, 12.5)
    q = np.full(n, 1e-9 / n)
    ax, ay, az = sc.relative_to_absolute(r[0], r[1], r[2], ref)
    want = [ref[d] + r[d].astype(np.float64) for d in range(3)]
    for a, w in zip((ax, ay, az), want):
        assert np.array_equal(a.cpu().numpy(), w)
    m = sc.Mesh3D((16, 16, 16), *want, precision="mixed")
    m.set_kick_mode("deterministic")  # bitwise reproducible rho: the two kicks must agree exactly
    e1 = sc.kick(m, ax, ay, az, q)
    e2 = sc.kick(m, *want, q)
    for a, b in zip(e1, e2):
        assert np.array_equal(a.cpu().numpy(), b)
