"""Velocity degree 3 (Q3-Q2, QGauss(4); the reference's degree-3 instantiation,
source/simulator/solver/stokes_matrix_free.cc:39-40,53-54) on the GPU against
the oracle (whose degree-3 operators are checked against dense assembly,
cubic reproduction of the transfers and the Q3 / Q2 convergence rates in
test_q3_cpu.py): every operator on every level (FP64 1e-12, FP32 2e-5),
diagonals, transfers, eigenvalue estimates, V-cycles and the block
preconditioner (1e-10), DGQ1 level tables, the rhs correction, and solves:
FP64-MG against the oracle's solution within 1e-8 with the same iteration
count (to one), the mixed-precision solve by the oracle's FP64 residual."""
import numpy as np
import pytest

from aspect_gb300 import gmg, mesh
from oracle import Oracle
from tests import numpy_reference as nr
from tests.gpu_util import p_err, random_eta, rel_err
from tests.test_q3_cpu import manufactured_problem

pytestmark = pytest.mark.gpu

CASES = [
    # dim, n, geometry, per_q, compressible
    (2, 8, "box", True, 0),
    (2, 8, "q2-distorted", False, 1),
    (3, 4, "box", False, 0),
    (3, 4, "box", True, 1),
    (3, 4, "table", True, 0),
]


def _levels(dim, n, geom):
    levels = mesh.box_hierarchy(dim, n, degree=3)
    if geom == "q2-distorted":
        levels = [mesh.to_q2_geometry(l, mesh.smooth_distortion()) for l in levels]
    elif geom == "table":
        levels = [mesh.to_table_geometry(mesh.to_q2_geometry(l, mesh.smooth_distortion())) for l in levels]
    return levels


def _eta(level, per_q, seed=1):
    rng = np.random.default_rng(seed)
    nq = 4 ** level.dim
    return np.exp(2.0 * rng.uniform(-1, 1, size=(level.n_cells, nq) if per_q else level.n_cells))


@pytest.fixture(scope="module", params=CASES, ids=lambda c: "-".join(map(str, c)))
def pair(request):
    dim, n, geom, per_q, comp = request.param
    levels = _levels(dim, n, geom)
    eta = _eta(levels[-1], per_q)
    g = gmg.StokesMatrixFreeGPU(dim, len(levels), degree=3)
    g.setup_dofs(levels)
    g.assemble(eta, 0, 1.9, comp)
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 1.9, comp)
    return levels, g, o


def test_q3_vmult_all_operators_all_levels(pair):
    levels, g, o = pair
    rng = np.random.default_rng(7)
    for lev, m in enumerate(levels):
        for op in range(4):
            n_in = m.n_u + m.n_p if op == 0 else (m.n_u if op == 1 else m.n_p)
            x = rng.normal(size=n_in)
            y_ref = o.vmult(op, lev, x)
            assert rel_err(g.vmult(op, lev, x, gmg.FP64), y_ref) < 1e-12, (lev, op)
            assert rel_err(g.vmult(op, lev, x, gmg.FP32), y_ref) < 2e-5, (lev, op)


def test_q3_diagonals_transfers_vcycles(pair):
    levels, g, o = pair
    g.build_preconditioner()
    o.build_preconditioner(False)
    for lev in range(len(levels)):
        for block in (0, 1):
            d_ref = o.diagonal_inverse(lev, block)
            assert rel_err(g.diagonal_inverse(lev, block, gmg.FP64), d_ref) < 1e-12, (lev, block)
            assert rel_err(g.diagonal_inverse(lev, block, gmg.FP32), d_ref) < 2e-5, (lev, block)
    rng = np.random.default_rng(3)
    for lev in range(1, len(levels)):
        for block in (0, 1):
            c, f = levels[lev - 1], levels[lev]
            xc = rng.normal(size=c.n_u if block == 0 else c.n_p)
            xf = rng.normal(size=f.n_u if block == 0 else f.n_p)
            assert rel_err(g.transfer(lev, block, False, xc), o.transfer(lev, block, False, xc)) < 1e-13
            assert rel_err(g.transfer(lev, block, True, xf), o.transfer(lev, block, True, xf)) < 1e-13
    o.estimate_eigenvalues()
    for lev in range(len(levels)):
        for block in (0, 1):
            e_ref = o.eigenvalues(lev, block)
            e64 = g.eigenvalues(lev, block, gmg.FP64)
            assert abs(e64[1] - e_ref[1]) < 1e-8 * abs(e_ref[1]), (lev, block, e64, e_ref)
            o.set_eigenvalues(lev, block, e64)
    f = levels[-1]
    for block in (0, 1):
        r = rng.normal(size=f.n_u if block == 0 else f.n_p)
        assert rel_err(g.vcycle(block, r, gmg.FP64), o.vcycle(block, r)) < 1e-10
    r = rng.normal(size=f.n_u + f.n_p)
    assert rel_err(g.block_preconditioner(r, gmg.FP64), o.block_preconditioner(r)) < 1e-10


@pytest.mark.parametrize("dim", [2, 3])
def test_q3_dgq1_level_tables(dim):
    levels = _levels(dim, 8 if dim == 2 else 4, "box")
    eta = _eta(levels[-1], True, seed=4)
    g = gmg.StokesMatrixFreeGPU(dim, len(levels), degree=3)
    g.setup_dofs(levels)
    g.assemble(eta, 1, 1.0)
    o = Oracle(levels)
    o.set_viscosity(eta, 1, 1.0)
    x = np.random.default_rng(2).normal(size=levels[-1].n_u)
    for lev in range(len(levels)):
        xl = x[: levels[lev].n_u]
        assert rel_err(g.vmult(gmg.OP_A, lev, xl, gmg.FP64), o.vmult(1, lev, xl)) < 1e-12, lev


def test_q3_correct_stokes_rhs():
    levels = _levels(2, 8, "q2-distorted")
    f = levels[-1]
    eta = _eta(f, True, seed=6)
    g = gmg.StokesMatrixFreeGPU(2, len(levels), degree=3)
    g.setup_dofs(levels)
    g.assemble(eta, 0, 1.4)
    rng = np.random.default_rng(11)
    mu = f.constraints_u.constrained_mask(f.n_u)
    u0 = np.zeros(f.n_u + f.n_p)
    u0[: f.n_u][mu] = rng.normal(size=mu.sum())
    rhs = rng.normal(size=f.n_u + f.n_p)
    got = g.correct_stokes_rhs(u0, rhs)
    A, BT, M = nr.stokes_blocks(f, eta, 1.4)
    K = np.block([[A, BT], [BT.T, np.zeros((f.n_p, f.n_p))]])
    C = np.zeros((f.n_u + f.n_p, f.n_u + f.n_p))
    C[: f.n_u, : f.n_u] = nr.constraint_matrix(f.n_u, f.constraints_u)
    C[f.n_u:, f.n_u:] = nr.constraint_matrix(f.n_p, f.constraints_p)
    assert rel_err(got - rhs, -(C.T @ (K @ u0))) < 1e-12


def test_q3_manufactured_solve_matches_oracle():
    levels, rhs = manufactured_problem(16, 3)
    f = levels[-1]
    eta = np.ones(f.n_cells)
    g = gmg.StokesMatrixFreeGPU(2, len(levels), degree=3)
    g.setup_dofs(levels)
    g.assemble(eta, 0, 1.0)
    g.build_preconditioner()
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 1.0)
    o.build_preconditioner(False)
    xo, io = o.solve(rhs, tol_rel=1e-10)
    x64, i64 = g.solve(rhs, linear_solver_tolerance=1e-10, mg_precision=gmg.FP64)
    assert abs(i64["cheap_iterations"] - io["cheap_iterations"]) <= 1, (i64, io)
    assert rel_err(x64[: f.n_u], xo[: f.n_u]) < 1e-8
    assert p_err(x64[f.n_u:], xo[f.n_u:]) < 1e-8
    x32, i32 = g.solve(rhs, linear_solver_tolerance=1e-10, mg_precision=gmg.FP32)
    r = np.linalg.norm(rhs - o.vmult(0, len(levels) - 1, x32))
    assert r <= 1.01 * i32["solver_tolerance"], (r, i32)


def test_q3_3d_variable_viscosity_solve():
    """3D 8^3 Q3-Q2 with a 1e3 viscosity contrast: FP64-MG against the oracle's
    solve, the mixed-precision solution by the oracle's FP64 residual."""
    levels = _levels(3, 8, "box")
    f = levels[-1]
    eta = _eta(f, False, seed=8) ** 1.5
    rng = np.random.default_rng(4)
    rhs = np.concatenate([rng.normal(size=f.n_u), np.zeros(f.n_p)])
    rhs[f.constraints_u.rows] = 0.0
    g = gmg.StokesMatrixFreeGPU(3, len(levels), degree=3)
    g.setup_dofs(levels)
    g.assemble(eta, 0, 1.0)
    g.build_preconditioner()
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 1.0)
    o.build_preconditioner(False)
    xo, io = o.solve(rhs, tol_rel=1e-8)
    x64, i64 = g.solve(rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP64)
    assert abs(i64["cheap_iterations"] - io["cheap_iterations"]) <= 1, (i64, io)
    assert rel_err(x64[: f.n_u], xo[: f.n_u]) < 1e-6
    x32, i32 = g.solve(rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    r = np.linalg.norm(rhs - o.vmult(0, len(levels) - 1, x32))
    assert r <= 1.01 * i32["solver_tolerance"], (r, i32)


def test_q3_degree_two_only_features_are_rejected():
    levels = _levels(2, 4, "box")
    g = gmg.StokesMatrixFreeGPU(2, len(levels), degree=3)
    g.setup_dofs(levels)
    g.assemble(np.ones(levels[-1].n_cells), 0, 1.0)
    f = levels[-1]
    with pytest.raises(gmg.GmgError):
        g.assemble_rhs(np.zeros((f.n_cells, 16, 2)))
    with pytest.raises(gmg.GmgError):
        g.adjoint_gradient(np.zeros(f.n_u), np.zeros(f.n_u))
    E = np.zeros((f.n_cells, 16, 3))
    with pytest.raises(gmg.GmgError):
        g.set_newton_terms(newton=True, strain_rate=E, d_eta_d_strain_rate=E, d_eta_d_pressure=E[..., 0])
