"""CPU oracle for the space-charge kick: TEST INFRASTRUCTURE ONLY.

This package restates SpaceCharge.jl's algorithm (src/mesh.jl, src/deposition.jl,
src/green_functions.jl, src/solvers/free_space.jl, src/interpolation.jl) in FP64
NumPy/SciPy, step by step and in the same order of operations, so that the
CUDA library can be checked against it.  It is imported only by `tests/`,
`__graft_entry__.smoke()` and the CPU-baseline leg of `bench.py`; the product
path (the C-ABI library and its Python/Julia hosts) never imports or calls it.

Parity status.  The reference ships no golden vectors and its Julia toolchain
is absent here, so the restatement cannot be run side by side with the
reference.  It is pinned instead against every known-answer fixture the
reference's own test suite holds for this path (test/test_mesh.jl,
test/test_deposition.jl, test/test_solvers.jl, test/test_interpolation.jl,
test/test_gpu.jl, test/analytical_test.jl), restated as tests in
tests/test_oracle.py, plus analytic known answers the reference's formulas must
satisfy (isotropic Gaussian field, cell-integrated Green function vs cubature,
Lorentz-boosted Gaussian, image charge).  Bit-level parity with FFTW 3.3.11
(FFTW_jll 3.3.11+0, the reference's CPU FFT) is unpinned: pocketfft (scipy)
stands in for it and agrees to ~1e-15 relative.
"""
from .sc_oracle import *  # noqa: F401,F403
