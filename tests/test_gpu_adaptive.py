"""Adaptive meshes with hanging nodes on the GPU (indexed layout, constraint
lines in the gathers, unchanged-cell transfers) against the CPU oracle, and the
adaptive-sphere workload (16^3 + 2 adaptive levels) solved in mixed and FP64
precision."""
import numpy as np
import pytest

from aspect_gb300 import gmg, octree, problems
from oracle import Oracle
from tests.gpu_util import p_err, rel_err

pytestmark = pytest.mark.gpu


def _pair(dim, base, nad, per_q):
    leaves = octree.sphere_refined_leaves(dim, base, nad, (0.5,) * dim, 0.2 if dim == 3 else 0.3)
    levels = octree.hierarchy(leaves, dim)
    f = levels[-1]
    rng = np.random.default_rng(9)
    eta = np.exp(2 * rng.uniform(-1, 1, size=(f.n_cells, 3 ** dim) if per_q else f.n_cells))
    g = gmg.StokesMatrixFreeGPU(dim, len(levels))
    g.setup_dofs(levels)
    g.assemble(eta, 0, 3.0)
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 3.0)
    return levels, g, o


@pytest.fixture(scope="module", params=[(2, 3, 2, True), (3, 2, 2, False), (3, 2, 1, True)],
                ids=lambda c: "-".join(map(str, c)))
def pair(request):
    return _pair(*request.param)


def test_adaptive_operators_diagonals_transfers(pair):
    levels, g, o = pair
    rng = np.random.default_rng(2)
    for lev, m in enumerate(levels):
        for op in range(4):
            n_in = m.n_u + m.n_p if op == 0 else (m.n_u if op == 1 else m.n_p)
            x = rng.normal(size=n_in)
            ref = o.vmult(op, lev, x)
            assert rel_err(g.vmult(op, lev, x, gmg.FP64), ref) < 1e-12, (lev, op)
            assert rel_err(g.vmult(op, lev, x, gmg.FP32), ref) < 2e-5, (lev, op)
    g.build_preconditioner()
    o.build_preconditioner(False)
    for lev in range(len(levels)):
        for block in (0, 1):
            assert rel_err(g.diagonal_inverse(lev, block), o.diagonal_inverse(lev, block)) < 1e-12
    for lev in range(1, len(levels)):
        c, f = levels[lev - 1], levels[lev]
        for block in (0, 1):
            xc = rng.normal(size=c.n_u if block == 0 else c.n_p)
            xf = rng.normal(size=f.n_u if block == 0 else f.n_p)
            assert rel_err(g.transfer(lev, block, False, xc), o.transfer(lev, block, False, xc)) < 1e-13
            assert rel_err(g.transfer(lev, block, True, xf), o.transfer(lev, block, True, xf)) < 1e-13


def test_adaptive_vcycles(pair):
    levels, g, o = pair
    g.build_preconditioner()
    o.build_preconditioner(False)
    for lev in range(len(levels)):
        for block in (0, 1):
            o.set_eigenvalues(lev, block, g.eigenvalues(lev, block, gmg.FP64))
    f = levels[-1]
    rng = np.random.default_rng(8)
    r = rng.normal(size=f.n_u + f.n_p)
    assert rel_err(g.block_preconditioner(r, gmg.FP64), o.block_preconditioner(r)) < 1e-10


@pytest.mark.parametrize("base,nad", [(3, 2), (4, 2)])
def test_adaptive_sphere_solve(base, nad):
    P = problems.adaptive_sphere(base, nad)
    g = gmg.from_problem(P)
    x64, o64 = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP64)
    x32, o32 = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    assert o64["status"] == 0 and o32["status"] == 0
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    top = len(P.levels) - 1
    for x, out in ((x64, o64), (x32, o32)):
        assert np.linalg.norm(P.rhs - o.vmult(0, top, x)) <= 1.01 * out["solver_tolerance"]
    f = P.fine
    # both meet the same FP64 residual; they agree to the problem's conditioning
    assert rel_err(x32[: f.n_u], x64[: f.n_u]) < 1e-5
    o.build_preconditioner(False)
    xr, info = o.solve(P.rhs, tol_rel=1e-8)
    assert abs(info["cheap_iterations"] - o64["cheap_iterations"]) <= 1
    assert rel_err(x64[: f.n_u], xr[: f.n_u]) < 1e-8 and p_err(x64[f.n_u:], xr[f.n_u:]) < 1e-8
