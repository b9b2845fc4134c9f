"""sc_solve_noalloc: the allocation-free solve for callers that cannot let a
library call cudaMalloc (a host code that owns all device memory through
its own pool, or a loop that forbids device allocation once running).

Through the C ABI it must give the same field as the regular entry point
(sc_solve on a mixed-precision mesh) and as the FP64 oracle, within the
mixed tolerance of the parity tests (1e-5 relative to the largest field
value), on two calls in a row with different grids and charges.  The second
call runs with the library's allocator set to fail every request and must
still succeed, and a warm call must leave the device's free memory
unchanged.  Grids beyond its fixed scratch are rejected with a clear error.
This file is collected last so that a run that stops at the first failure
has run every other test before it."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bunch(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.standard_normal((3, n)).clip(-4.5, 4.5)
    return v[0] * 1e-3, v[1] * 0.7e-3, v[2] * 0.3e-3


def _noalloc(L, grid, delta, gamma, rho, out, stream):
    L.call("sc_solve_noalloc", (C.c_int32 * 3)(*grid), (C.c_double * 3)(*delta), float(gamma),
           C.c_void_p(rho.data_ptr()), C.c_void_p(out.data_ptr()), stream)


def test_noalloc_matches_solve_twice(sc, lib, cuda):
    import torch

    import oracle as O
    from spacecharge_gb300 import _lib as L

    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    cases = (((16, 16, 24), 3.0, 1), ((32, 20, 9), 1.0, 2))
    for i, (grid, gamma, seed) in enumerate(cases):
        x, y, z = _bunch(20000, seed)
        q = np.full(x.size, 1e-9 / x.size)
        lo, hi = (-5e-3, -3.5e-3, -1.5e-3), (5e-3, 3.5e-3, 1.5e-3)
        m = sc.Mesh3D(grid, lo, hi, precision="mixed", gamma=gamma)
        sc.deposit(m, x, y, z, q)
        sc.solve(m)
        ref = m.efield.detach().clone()
        nx, ny, nz = grid
        out = torch.full((nz, ny, nx, 4), float("nan"), dtype=torch.float32, device="cuda")
        rho = m.rho.permute(2, 1, 0).contiguous()  # (nz, ny, nx) = x fastest
        torch.cuda.synchronize()
        if i == 0:
            _noalloc(L, grid, m.delta, gamma, rho, out, stream)
        else:
            # the library's allocator fails every request: the call must not need one
            free0 = torch.cuda.mem_get_info()[0]
            lib.sc_test_fail_allocations(0)
            try:
                _noalloc(L, grid, m.delta, gamma, rho, out, stream)
            finally:
                lib.sc_test_fail_allocations(-1)
            torch.cuda.synchronize()
            assert torch.cuda.mem_get_info()[0] == free0
        torch.cuda.synchronize()
        got = out.permute(2, 1, 0, 3)[..., :3]
        assert torch.isfinite(got).all()
        scale = ref.abs().max().item()
        assert scale > 0
        err = (got - ref).abs().max().item() / scale
        assert err <= 1e-5, (grid, err)
        # the FP64 oracle on the same bounds and charges
        om = O.mesh_manual(grid, lo, hi, gamma=gamma)
        O.deposit(om, x, y, z, q)
        O.solve(om)
        oe = om.efield
        got_np = got.double().cpu().numpy()
        err_o = np.abs(got_np - oe).max() / np.abs(oe).max()
        assert err_o <= 1e-5, (grid, err_o)


def test_noalloc_rejects_large_grid(sc, cuda):
    import torch

    from spacecharge_gb300 import _lib as L

    buf = torch.zeros(4 * 33 * 8 * 8, dtype=torch.float32, device="cuda")
    with pytest.raises(sc.SpaceChargeError, match="at most 32 nodes per axis"):
        L.call("sc_solve_noalloc", (C.c_int32 * 3)(33, 8, 8), (C.c_double * 3)(1e-4, 1e-4, 1e-4), 1.0,
               C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()), None)
