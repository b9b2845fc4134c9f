"""GB300 space-charge kick: Python host of libspacecharge_gb300.so.

Mirrors SpaceCharge.jl's exports (src/SpaceCharge.jl:17): Mesh3D, deposit
(deposit!), clear_mesh (clear_mesh!), interpolate_field, solve (solve!), plus
kick (the three in one library call).
"""
from ._lib import SpaceChargeError, load  # noqa: F401
from .mesh import (CLIGHT, FPEI, Batch, Mesh3D, autotune, clear_mesh, deposit, interpolate_field, kick,  # noqa: F401
                   kick_adjoint, kick_autograd, kick_host, solve, magnetic_field, aos_to_soa, soa_to_aos,
                   relative_to_absolute, solve_potential, track)

__all__ = ["Mesh3D", "deposit", "clear_mesh", "interpolate_field", "solve", "kick", "kick_host", "kick_adjoint",
           "kick_autograd", "Batch", "autotune", "SpaceChargeError", "magnetic_field", "aos_to_soa",
           "soa_to_aos", "relative_to_absolute", "solve_potential", "track",
           "CLIGHT", "FPEI", "load"]
