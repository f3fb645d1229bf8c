"""Spherical shell on the GPU: curved Q2 cells (per-point geometry tables),
no-normal-flux lines coupling velocity components, parity with the oracle; and
the shell workload (96-cell cube-sphere refined 3 times, ~1.2M DoFs, free slip
on both spheres) solved with the FP64 dense coarse solve in mixed and FP64
precision, each residual checked by the oracle in FP64."""
import numpy as np
import pytest

from aspect_gb300 import gmg, problems, shell
from oracle import Oracle
from tests.gpu_util import rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pair():
    levels = shell.hierarchy(1)
    f = levels[-1]
    rng = np.random.default_rng(5)
    eta = np.exp(rng.uniform(-2, 2, size=(f.n_cells, 27)))
    g = gmg.StokesMatrixFreeGPU(3, len(levels))
    g.setup_dofs(levels)
    g.assemble(eta, 0, 2.0)
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 2.0)
    return levels, g, o


def test_shell_parity(pair):
    levels, g, o = pair
    rng = np.random.default_rng(1)
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
            o.set_eigenvalues(lev, block, g.eigenvalues(lev, block, gmg.FP64))
    f = levels[-1]
    xf = rng.normal(size=f.n_u)
    assert rel_err(g.transfer(1, 0, True, xf), o.transfer(1, 0, True, xf)) < 1e-13
    r = rng.normal(size=f.n_u + f.n_p)
    assert rel_err(g.block_preconditioner(r, gmg.FP64), o.block_preconditioner(r)) < 1e-10


def _emulated_vcycle(g, levels, r, coarse):
    """The velocity V-cycle (Chebyshev degree 4, range 15, one step; coarse solve
    given as a function) written out in numpy over the solver's own level
    operators, transfers, diagonals and eigenvalue estimates."""
    def cheb(lev, x, b):
        emin, emax = g.eigenvalues(lev, 0, gmg.FP64)
        lmax = 1.2 * emax
        alpha = lmax / 15.0
        theta, delta = 0.5 * (lmax + alpha), 0.5 * (lmax - alpha)
        dinv = g.diagonal_inverse(lev, 0)
        if x is None:
            d = dinv * b / theta
            x = d.copy()
        else:
            d = dinv * (b - g.vmult(1, lev, x, gmg.FP64)) / theta
            x = x + d
        rhok, sigma = delta / theta, theta / delta
        for _ in range(1, 4):
            rhokp = 1.0 / (2.0 * sigma - rhok)
            d = rhokp * rhok * d + 2.0 * rhokp / delta * dinv * (b - g.vmult(1, lev, x, gmg.FP64))
            rhok = rhokp
            x = x + d
        return x

    def level(lev, b):
        if lev == 0:
            return coarse(b)
        x = cheb(lev, None, b)
        c = g.transfer(lev, 0, True, b - g.vmult(1, lev, x, gmg.FP64))
        x = x + g.transfer(lev, 0, False, level(lev - 1, c))
        return cheb(lev, x, b)

    return level(len(levels) - 1, r)


def test_dense_coarse_vcycle_three_levels():
    """A three-level V-cycle with the FP64 dense coarse solve equals the same
    cycle written out in numpy with numpy's pseudo-inverse of the level-0 matrix
    (assembled column by column from the solver's level operator)."""
    P = problems.spherical_shell(2)
    g = gmg.from_problem(P, options={"coarse_solver": gmg.COARSE_DENSE_FP64})
    n0 = P.levels[0].n_u
    M = np.zeros((n0, n0))
    for j in range(n0):
        e = np.zeros(n0)
        e[j] = 1.0
        M[:, j] = g.vmult(1, 0, e, gmg.FP64)
    pinv = np.linalg.pinv(0.5 * (M + M.T), rcond=1e-10, hermitian=True)
    r = np.random.default_rng(7).normal(size=P.fine.n_u)
    ref = _emulated_vcycle(g, P.levels, r, lambda b: pinv @ b)
    assert rel_err(g.vcycle(0, r, gmg.FP64), ref) < 1e-9
    assert rel_err(g.vcycle(0, r, gmg.FP32), ref) < 1e-4


def _remove_rotations(level, u):
    modes = shell.rotation_modes(level)
    q, _ = np.linalg.qr(modes.T)
    return u - q @ (q.T @ u)


@pytest.mark.parametrize("n_ref", [2, 3])
def test_shell_solve_dense_coarse(n_ref):
    P = problems.spherical_shell(n_ref)
    g = gmg.from_problem(P, options={"coarse_solver": gmg.COARSE_DENSE_FP64})
    x32, o32 = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    x64, o64 = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP64)
    assert o32["status"] == 0 and o64["status"] == 0
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    top = len(P.levels) - 1
    for x, out in ((x32, o32), (x64, o64)):
        assert np.linalg.norm(P.rhs - o.vmult(0, top, x)) <= 1.01 * out["solver_tolerance"]
    f = P.fine
    u32 = _remove_rotations(f, x32[: f.n_u])
    u64 = _remove_rotations(f, x64[: f.n_u])
    assert rel_err(u32, u64) < 1e-5


@pytest.fixture(scope="module")
def adaptive_pair():
    """Shell refined once globally plus one round on the temperature gradient:
    curved cells of two depths, hanging-node lines (Q2 velocity, Q1 pressure)
    across patch boundaries, no-normal-flux lines on hanging boundary nodes, and
    transfers with cells that are their own parent."""
    P = problems.spherical_shell(1, n_adaptive=1)
    levels = P.levels
    f = levels[-1]
    rng = np.random.default_rng(6)
    eta = np.exp(rng.uniform(-2, 2, size=(f.n_cells, 27)))
    g = gmg.StokesMatrixFreeGPU(3, len(levels))
    g.setup_dofs(levels)
    g.assemble(eta, 0, 2.0)
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 2.0)
    return levels, g, o


def test_adaptive_shell_parity(adaptive_pair):
    levels, g, o = adaptive_pair
    assert levels[-1].constraints_p.n_lines > 0
    test_shell_parity(adaptive_pair)
    f = levels[-1]
    rng = np.random.default_rng(2)
    xc = rng.normal(size=levels[-2].n_u)
    assert rel_err(g.transfer(len(levels) - 1, 0, False, xc), o.transfer(len(levels) - 1, 0, False, xc)) < 1e-13
    xp = rng.normal(size=f.n_p)
    assert rel_err(g.transfer(len(levels) - 1, 1, True, xp), o.transfer(len(levels) - 1, 1, True, xp)) < 1e-13


def test_adaptive_shell_solve_dense_coarse():
    """The shell workload's adaptive form at reduced size (refinement 2 plus one
    round on the temperature gradient), FP64 dense coarse solve, mixed and FP64
    precision; residuals checked by the oracle in FP64. With hanging nodes the
    rigid rotations are no longer exact null vectors (the fine nodes lie on the
    spheres, the coarse faces are Q2 interpolants), so velocities are compared
    after removing them."""
    P = problems.spherical_shell(2, n_adaptive=1)
    g = gmg.from_problem(P, options={"coarse_solver": gmg.COARSE_DENSE_FP64})
    x32, o32 = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    x64, o64 = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP64)
    assert o32["status"] == 0 and o64["status"] == 0, (o32, o64)
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    top = len(P.levels) - 1
    for x, out in ((x32, o32), (x64, o64)):
        assert np.linalg.norm(P.rhs - o.vmult(0, top, x)) <= 1.01 * out["solver_tolerance"]
    f = P.fine
    assert rel_err(_remove_rotations(f, x32[: f.n_u]), _remove_rotations(f, x64[: f.n_u])) < 1e-4
