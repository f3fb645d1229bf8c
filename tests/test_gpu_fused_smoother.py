"""Fused small-level A-block smoother (gb_gmg_options.fused_small_smoother): each
Chebyshev step's gather and the next cell pass in one launch on the small 3D
lattice levels. The same arithmetic as the two-launch steps, so on the same
handle data the FP32 velocity V-cycle, the block preconditioner and a mixed
solve equal those of the unfused smoother (bit for bit where the compiler
forms the same products; checked at 1e-7 relative), with the explicit coarse
sub-cycle (only the 8^3 level fused) and without it (levels 1 to 3 fused), for
per-cell and per-point viscosity tables, no-slip and free-slip faces."""
import numpy as np
import pytest

from aspect_gb300 import gmg, problems
from tests.gpu_util import p_err, rel_err

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,dense,projection", [(32, 2200, 1), (16, 0, 1), (16, 0, 0)])
def test_fused_small_smoother_equals_two_launch_steps(n, dense, projection):
    P = problems.sinkers_3d(n, projection=projection)
    on = gmg.from_problem(P, {"dense_a_cycle_dofs": dense})
    off = gmg.from_problem(P, {"dense_a_cycle_dofs": dense, "fused_small_smoother": 0})
    f = P.fine
    rng = np.random.default_rng(5)
    for _ in range(2):
        r = rng.normal(size=f.n_u)
        assert rel_err(on.vcycle(0, r, gmg.FP32), off.vcycle(0, r, gmg.FP32)) < 1e-7
    r = rng.normal(size=f.n_u + f.n_p)
    assert rel_err(on.block_preconditioner(r, gmg.FP32), off.block_preconditioner(r, gmg.FP32)) < 1e-7
    # FP64 V-cycles never take the fused path
    assert rel_err(on.vcycle(0, r[: f.n_u], gmg.FP64), off.vcycle(0, r[: f.n_u], gmg.FP64)) == 0.0
    xa, oa = on.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    xb, ob = off.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    assert oa["status"] == 0 and ob["status"] == 0
    assert oa["cheap_iterations"] == ob["cheap_iterations"]
    assert rel_err(xa[: f.n_u], xb[: f.n_u]) < 1e-10
    assert p_err(xa[f.n_u:], xb[f.n_u:]) < 1e-8


def test_fused_small_smoother_free_slip_2d_unaffected():
    """2D levels keep the two-launch steps (the small-level kernel is 3D): the
    option changes nothing there."""
    P = problems.solcx(5)
    on = gmg.from_problem(P)
    off = gmg.from_problem(P, {"fused_small_smoother": 0})
    r = np.random.default_rng(2).normal(size=P.fine.n_u)
    assert rel_err(on.vcycle(0, r, gmg.FP32), off.vcycle(0, r, gmg.FP32)) == 0.0
