"""IDR(s) as the cheap Krylov method (the reference's "Krylov method for cheap
solver steps = IDR(s)"), on the CPU oracle: converged solves whose true FP64
residual meets the tolerance, with the iteration structure of the reference's
IDR(2) output (s + 1 preconditioner applications per iteration, the last one
ending after its first converged residual update). The reference's own IDR(2)
numbers on its NSinker test are pinned in test_oracle_pins.py."""
import numpy as np
import pytest

from aspect_gb300 import problems
from oracle import Oracle


@pytest.mark.parametrize("name,s", [("solcx", 1), ("solcx", 2), ("solcx", 4), ("sinkers", 2)])
def test_oracle_idr_converges_with_reference_iteration_structure(name, s):
    P = problems.solcx(4) if name == "solcx" else problems.sinkers_3d(4)
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    o.build_preconditioner(False)
    x, info = o.solve(P.rhs, tol_rel=1e-8, krylov=2, idr_s=s)
    assert info["status"] == 0 and info["expensive_iterations"] == 0
    r = P.rhs - o.vmult(0, len(P.levels) - 1, x)
    assert np.linalg.norm(r) <= info["solver_tolerance"]
    its, na = info["cheap_iterations"], info["A_preconditioner_applications"]
    assert (s + 1) * (its - 1) + 1 <= na <= (s + 1) * its
    # same solution as GMRES within the conditioning of a 1e-8 residual
    xg, ig = o.solve(P.rhs, tol_rel=1e-8)
    f = P.fine
    assert np.linalg.norm(x[: f.n_u] - xg[: f.n_u]) <= 1e-5 * np.linalg.norm(xg[: f.n_u])


def test_oracle_idr_with_fp32_vcycles_reaches_the_true_residual():
    """FP32 V-cycles are not exactly linear; IDR(s) still ends on the true FP64
    residual (restarting from it if the recursively updated one has drifted),
    here at a 1e-10 relative tolerance."""
    P = problems.sinkers_3d(8)
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    o.build_preconditioner(True)
    x, info = o.solve(P.rhs, tol_rel=1e-10, krylov=2, idr_s=2)
    assert info["status"] == 0 and info["expensive_iterations"] == 0
    r = P.rhs - o.vmult(0, len(P.levels) - 1, x)
    assert np.linalg.norm(r) <= info["solver_tolerance"]
