"""The far-cell rule of the mixed-precision Green build holds for cells of
any shape the workloads produce.

The mixed build (spacecharge.jl_gb300/csrc/native.cu, k_igf_split) replaces
the reference's FP64 8-point difference of the antiderivative
(src/green_functions.jl:35-38, 103-112) by Gauss-Legendre quadrature of
(u, v, w) / r^3 over the cell for cells whose centre lies at least
kNearRatio half-widths from the origin, with 4, 3 or 2 points per axis as
R / hmax grows (hmax = half of the longest cell width, so boosted cells
gamma * dz long count by their long side).  This restates that rule in FP64
NumPy and checks its truncation error against a 16-point rule over cell
aspect ratios from 1/500 to 500 (dz_boosted / dx; 500 is the most elongated
bunch of the 64-bunch workload).  The thresholds are read from native.cu so
the test follows the kernel's constants.
"""
from __future__ import annotations

import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "spacecharge.jl_gb300", "csrc", "native.cu")


def _constants():
    text = open(SRC, encoding="utf-8").read()
    out = {}
    for name in ("kNearRatio", "kQ3Ratio", "kQ2Ratio"):
        m = re.search(rf"constexpr double {name} = ([0-9.]+);", text)
        assert m, name
        out[name] = float(m.group(1))
    return out


def _cell_integral(c, h, n):
    """sum over an n^3 Gauss-Legendre rule of w_i w_j w_k p / |p|^3 with p
    the quadrature points of the cell centred at c (3, M) with half-widths
    h; the 1/8 Jacobian factor is common to every rule and left out."""
    t, w = np.polynomial.legendre.leggauss(n)
    px = c[0][:, None, None, None] + h[0] * t[None, :, None, None]
    py = c[1][:, None, None, None] + h[1] * t[None, None, :, None]
    pz = c[2][:, None, None, None] + h[2] * t[None, None, None, :]
    W = w[:, None, None] * w[None, :, None] * w[None, None, :]
    ir = 1.0 / np.sqrt(px * px + py * py + pz * pz)
    q = W[None] * ir ** 3
    return np.stack([(q * px).sum((1, 2, 3)), (q * py).sum((1, 2, 3)), (q * pz).sum((1, 2, 3))])


@pytest.mark.parametrize("aspect", [1.0, 5.0, 100.0, 500.0, 0.2, 1 / 100, 1 / 500])
def test_far_cell_quadrature_truncation(aspect):
    k = _constants()
    # cell widths in units of hmax (the longest is 2)
    u = (2 / aspect, 2 / aspect, 2.0) if aspect >= 1 else (2.0, 2.0, 2 * aspect)
    h = tuple(v / 2 for v in u)
    rng = np.random.default_rng(0)
    reach = 3 * k["kQ2Ratio"]
    idx = [rng.integers(0, int(reach / u[d]) + 2, 40000) for d in range(3)]
    c = np.array([idx[d] * u[d] for d in range(3)], dtype=np.float64)
    R = np.sqrt((c ** 2).sum(0))
    c, R = c[:, R >= k["kNearRatio"]], R[R >= k["kNearRatio"]]
    bands = [(4, R < k["kQ3Ratio"]), (3, (R >= k["kQ3Ratio"]) & (R < k["kQ2Ratio"])), (2, R >= k["kQ2Ratio"])]
    # every band, the closest cells of each band included
    for n, sel in bands:
        cs = c[:, sel]
        order = np.argsort(R[sel])
        cs = np.concatenate([cs[:, order[:2000]], cs[:, order[-500:]]], axis=1)
        ref = _cell_integral(cs, h, 16)
        got = _cell_integral(cs, h, n)
        err = np.sqrt(((got - ref) ** 2).sum(0)) / np.sqrt((ref ** 2).sum(0))
        # below FP32 rounding of the sums themselves (~3e-7), far below the
        # 1e-5 field tolerance
        assert err.max() < 2.5e-7, (aspect, n, float(err.max()))
