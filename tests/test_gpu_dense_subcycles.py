"""The coarse sub-cycles of the FP32 V-cycles as explicit matrices
(options dense_mass_cycle_nodes / dense_a_cycle_dofs) against the multi-launch
cycles they replace, on the same handle data: the FP32 V-cycles of both blocks
agree to FP32 rounding (1e-5 relative, the tolerance of the FP32-vs-FP64
V-cycle tests); the matrices follow a change of the FP32 eigenvalue estimates
of their levels (gb_gmg_set_eigenvalues) and of the viscosity
(gb_gmg_update_viscosity); and a mixed solve takes the same iterations with
and without them, to solutions within 1e-8."""
import numpy as np
import pytest

from aspect_gb300 import gmg, problems
from tests.gpu_util import random_eta, rel_err

pytestmark = pytest.mark.gpu

OFF = {"dense_mass_cycle_nodes": 0, "dense_a_cycle_dofs": 0}


def _pair(n=16, projection=1):
    P = problems.sinkers_3d(n, projection=projection)
    on = gmg.from_problem(P)
    off = gmg.from_problem(P, OFF)
    return P, on, off


@pytest.mark.parametrize("projection", [0, 1])
def test_dense_subcycles_equal_the_multi_launch_cycles(projection):
    P, on, off = _pair(16, projection)
    f = P.fine
    rng = np.random.default_rng(3)
    for block, n in ((0, f.n_u), (1, f.n_p)):
        r = rng.normal(size=n)
        a, b = on.vcycle(block, r, gmg.FP32), off.vcycle(block, r, gmg.FP32)
        assert rel_err(a, b) < 1e-5, (block, rel_err(a, b))
        assert rel_err(on.vcycle(block, r, gmg.FP64), off.vcycle(block, r, gmg.FP64)) == 0.0


def test_dense_subcycles_follow_eigenvalue_and_viscosity_changes():
    P, on, off = _pair(16, 1)
    f = P.fine
    rng = np.random.default_rng(5)
    # new FP32 intervals on the coarse levels of both blocks, the same on both handles
    for lev in range(3):
        for block in (0, 1):
            e = on.eigenvalues(lev, block, gmg.FP32) * np.array([1.0, 1.3])
            on.set_eigenvalues(lev, block, gmg.FP32, e)
            off.set_eigenvalues(lev, block, gmg.FP32, e)
    for block, n in ((0, f.n_u), (1, f.n_p)):
        r = rng.normal(size=n)
        assert rel_err(on.vcycle(block, r, gmg.FP32), off.vcycle(block, r, gmg.FP32)) < 1e-5, block
    # a new viscosity with the last-built preconditioner
    eta2 = P.eta * np.exp(0.5 * rng.uniform(-1, 1, size=P.eta.shape))
    on.update_viscosity(eta2)
    off.update_viscosity(eta2)
    for block, n in ((0, f.n_u), (1, f.n_p)):
        r = rng.normal(size=n)
        assert rel_err(on.vcycle(block, r, gmg.FP32), off.vcycle(block, r, gmg.FP32)) < 1e-5, block


def test_next_level_dense_subcycle():
    """dense_mass_cycle_nodes = 6000: the Schur sub-cycle matrix of the 16^3 level,
    built from the 8^3 level's by the batched steps, against the multi-launch cycle
    (32^3 hierarchy: the 16^3 level is below the top)."""
    P = problems.sinkers_3d(32, projection=1)
    wide = gmg.from_problem(P, {"dense_mass_cycle_nodes": 6000})
    off = gmg.from_problem(P, OFF)
    f = P.fine
    r = np.random.default_rng(8).normal(size=f.n_p)
    assert rel_err(wide.vcycle(1, r, gmg.FP32), off.vcycle(1, r, gmg.FP32)) < 1e-5


def test_mixed_solve_with_and_without_dense_subcycles():
    P, on, off = _pair(16, 1)
    f = P.fine
    xa, oa = on.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    xb, ob = off.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    assert oa["status"] == 0 and ob["status"] == 0
    assert oa["cheap_iterations"] == ob["cheap_iterations"]
    assert rel_err(xa[: f.n_u], xb[: f.n_u]) < 1e-8
