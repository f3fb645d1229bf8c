"""End-to-end solves on the GPU: the reference's SolCx regression outputs
(iteration counts and error norms of tests/sol_cx_{2,4}_gmg) and mixed-precision
solves against the FP64 oracle."""
import json
import os

import numpy as np
import pytest

from aspect_gb300 import gmg, problems
from oracle import Oracle
from tests.gpu_util import p_err, rel_err

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("nref", [2, 4])
def test_solcx_reference_regression_on_gpu(nref):
    golden = json.load(open(os.path.join(GOLDEN, "solcx_golden.json")))[str(2 ** nref)]
    exact = np.load(os.path.join(GOLDEN, "solcx_exact.npz"))
    P = problems.solcx(nref)
    g = gmg.from_problem(P)
    x, out = g.solve(P.rhs, linear_solver_tolerance=1e-7, mg_precision=gmg.FP64)
    assert out["status"] == 0
    assert out["cheap_iterations"] == golden["cheap_iterations"]
    f = P.fine
    u = x[: f.n_u].copy()
    p = x[f.n_u:] * P.pressure_scaling
    f.constraints_u.distribute(u)
    problems.normalize_pressure_surface(f, p)
    n = 2 ** nref
    errs = problems.error_norms(f, u, p, exact[f"u_{n}"], exact[f"p_{n}"])
    np.testing.assert_allclose(errs, golden["errors"], rtol=2e-6)


@pytest.mark.parametrize("precision", [gmg.FP64, gmg.FP32])
def test_solcx_64_matches_oracle(precision):
    P = problems.solcx(6, density_sign=1.0)
    g = gmg.from_problem(P)
    x, out = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=precision)
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    o.build_preconditioner(False)
    xr, info = o.solve(P.rhs, tol_rel=1e-8)
    f = P.fine
    assert out["status"] == 0 and info["status"] == 0
    # FP64: the same algorithm to rounding (1e-8); FP32 V-cycle: both satisfy the
    # same 1e-8 FP64 residual and agree to the conditioning
    tol = 1e-8 if precision == gmg.FP64 else 1e-6
    assert rel_err(x[: f.n_u], xr[: f.n_u]) < tol
    assert p_err(x[f.n_u:], xr[f.n_u:]) < tol
    if precision == gmg.FP64:
        assert abs(out["cheap_iterations"] - info["cheap_iterations"]) <= 1
    # true residual of the GPU solution, measured by the oracle in FP64
    r = P.rhs - o.vmult(0, len(P.levels) - 1, x)
    assert np.linalg.norm(r) <= 1.01 * out["solver_tolerance"]


@pytest.mark.parametrize("krylov", [gmg.GMRES, gmg.GMRES_IR])
def test_sinkers_mixed_precision(krylov):
    P = problems.sinkers_3d(8)
    g = gmg.from_problem(P)
    x64, o64 = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP64)
    x32, o32 = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32, krylov=krylov)
    assert o64["status"] == 0 and o32["status"] == 0
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    r = P.rhs - o.vmult(0, len(P.levels) - 1, x32)
    assert np.linalg.norm(r) <= 1.01 * o32["solver_tolerance"]
    f = P.fine
    assert rel_err(x32[: f.n_u], x64[: f.n_u]) < 1e-6
    assert p_err(x32[f.n_u:], x64[f.n_u:]) < 1e-6


def test_no_convergence_is_reported():
    """stokes_solver_fail_gmg: an unreachable tolerance ends in NO_CONVERGENCE."""
    P = problems.solcx(2)
    g = gmg.from_problem(P)
    with pytest.raises(gmg.NoConvergence):
        g.solve(P.rhs, absolute_tolerance=1e-300, n_cheap_steps=5, n_expensive_steps=3)


def test_solve_is_bit_reproducible():
    """Every reduction has a fixed summation order (the last-arriving block of a
    reduction sums the per-block partials in block order), so repeated mixed-
    precision solves give bit-identical solutions and iteration counts."""
    P = problems.sinkers_3d(8)
    g = gmg.from_problem(P)
    x1, o1 = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    x2, o2 = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    assert o1["cheap_iterations"] == o2["cheap_iterations"]
    assert np.array_equal(x1, x2)


@pytest.mark.parametrize("precision", [gmg.FP64, gmg.FP32])
def test_idr_matches_oracle(precision):
    """IDR(2) as the cheap Krylov method: same shadow space as the oracle (built
    in the caller's numbering), converged on the true FP64 residual; in FP64 the
    iteration count matches the oracle's within one."""
    P = problems.sinkers_3d(8)
    g = gmg.from_problem(P)
    x, out = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=precision, krylov=gmg.IDR, idr_s=2)
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    o.build_preconditioner(False)
    xr, info = o.solve(P.rhs, tol_rel=1e-8, krylov=2, idr_s=2)
    assert out["status"] == 0 and out["expensive_iterations"] == 0 and info["status"] == 0
    r = P.rhs - o.vmult(0, len(P.levels) - 1, x)
    assert np.linalg.norm(r) <= 1.01 * out["solver_tolerance"]
    f = P.fine
    tol = 1e-8 if precision == gmg.FP64 else 1e-6
    assert rel_err(x[: f.n_u], xr[: f.n_u]) < tol
    assert p_err(x[f.n_u:], xr[f.n_u:]) < tol
    if precision == gmg.FP64:
        assert abs(out["cheap_iterations"] - info["cheap_iterations"]) <= 1
