"""Velocity degree 3 (Q3-Q2, QGauss(4); the reference's degree-3 instantiation,
source/simulator/solver/stokes_matrix_free.cc:39-40,53-54, its test
tests/hollow_sphere_gmg_q3.prm) in the oracle, checked against the mathematics:
(1) every operator and the diagonals against dense matrices assembled in numpy
from the bilinear forms (per-cell and per-point viscosity, compressible,
distorted Q2 geometry); (2) the transfer reproduces cubic velocity and quadratic
pressure fields exactly; (3) a manufactured smooth solution converges at the
element's rates: velocity L2 error / 16 (Q3) and pressure / 8 (Q2) per halving
of h, against / 8 and / 4 for Q2-Q1."""
import numpy as np
import pytest

from aspect_gb300 import fe, mesh, problems
from oracle import Oracle
from tests import numpy_reference as nr


def _levels(dim, n, distorted=False):
    levels = mesh.box_hierarchy(dim, n, degree=3)
    if distorted:
        levels = [mesh.to_q2_geometry(l, mesh.smooth_distortion()) for l in levels]
    return levels


@pytest.mark.parametrize("dim,n,distorted,per_q,comp", [(2, 4, False, True, 0), (2, 4, True, False, 1),
                                                       (3, 2, False, True, 0), (3, 2, True, True, 1)])
def test_q3_oracle_operators_match_assembled(dim, n, distorted, per_q, comp):
    levels = _levels(dim, n, distorted)
    f = levels[-1]
    assert f.degree == 3 and f.cell_dofs_u.shape[1] == dim * 4 ** dim and f.cell_dofs_p.shape[1] == 3 ** dim
    rng = np.random.default_rng(3)
    nq = 4 ** dim
    eta = np.exp(rng.normal(size=(f.n_cells, nq) if per_q else f.n_cells))
    s = 2.3
    o = Oracle(levels)
    o.set_viscosity(eta, 0, s, comp)
    eq = eta if per_q else np.repeat(eta[:, None], nq, 1)
    A, BT, M = nr.stokes_blocks(f, eq, s, compressible=bool(comp))
    Cu = nr.constraint_matrix(f.n_u, f.constraints_u)
    mu = f.constraints_u.constrained_mask(f.n_u)
    Ac = nr.constrained_operator(A, Cu, Cu, mu)
    x = rng.normal(size=f.n_u + f.n_p)
    top = len(levels) - 1
    ya = o.vmult(1, top, x[: f.n_u])
    np.testing.assert_allclose(ya, Ac @ x[: f.n_u], rtol=1e-11, atol=1e-11 * np.abs(ya).max())
    ym = o.vmult(3, top, x[f.n_u:])
    np.testing.assert_allclose(ym, M @ x[f.n_u:], rtol=1e-11, atol=1e-11 * np.abs(ym).max())
    BTc = Cu.T @ BT
    BTc[mu, :] = 0
    K = np.block([[Ac, BTc], [BTc.T, np.zeros((f.n_p, f.n_p))]])
    ys = o.vmult(0, top, x)
    np.testing.assert_allclose(ys, K @ x, rtol=1e-11, atol=1e-11 * np.abs(ys).max())
    o.build_preconditioner(False)
    np.testing.assert_allclose(o.diagonal_inverse(top, 0), 1.0 / np.where(mu, 1.0, np.diag(Ac)), rtol=1e-11)
    np.testing.assert_allclose(o.diagonal_inverse(top, 1), 1.0 / np.diag(M), rtol=1e-11)


@pytest.mark.parametrize("dim", [2, 3])
def test_q3_transfer_reproduces_cubics(dim):
    levels = mesh.box_hierarchy(dim, 4, free_slip=False, degree=3)
    o = Oracle(levels)
    c, f = levels[-2], levels[-1]

    def field(x, comp):
        return 1 + x[:, 0] ** 3 - 0.5 * x[:, 1] ** 2 * (comp + 1) * x[:, 0] + (x[:, -1] ** 3 if dim == 3 else 0)

    uf = o.transfer(len(levels) - 1, 0, False, field(c.dof_points_u, c.dof_component_u))
    np.testing.assert_allclose(uf, field(f.dof_points_u, f.dof_component_u), rtol=1e-12, atol=1e-12)
    pc = 1 + c.dof_points_p[:, 0] ** 2 - c.dof_points_p[:, 1] * c.dof_points_p[:, -1]
    pf = o.transfer(len(levels) - 1, 1, False, pc)
    np.testing.assert_allclose(pf, 1 + f.dof_points_p[:, 0] ** 2 - f.dof_points_p[:, 1] * f.dof_points_p[:, -1],
                               rtol=1e-12, atol=1e-12)


def manufactured_problem(n, degree):
    """u = (sin pi x cos pi y, -cos pi x sin pi y), p = cos pi x cos pi y, eta = 1 on
    the unit square with free slip (exactly satisfied: u.n = 0 and eps_nt = 0 on
    the walls): f = -div(2 eps(u)) + grad p = 2 pi^2 u + grad p."""
    levels = mesh.box_hierarchy(2, n, degree=degree)
    f = levels[-1]
    xq, _ = problems.q_points_real(f, degree + 1)
    x, y = xq[..., 0], xq[..., 1]
    pi = np.pi
    force = np.stack([2 * pi ** 2 * np.sin(pi * x) * np.cos(pi * y) - pi * np.sin(pi * x) * np.cos(pi * y),
                      -2 * pi ** 2 * np.cos(pi * x) * np.sin(pi * y) - pi * np.cos(pi * x) * np.sin(pi * y)], -1)
    rhs = problems.assemble_rhs(f, force)
    return levels, rhs


def exact_errors(level, u, p):
    xq, _ = problems.q_points_real(level, 6)
    x, y = xq[..., 0], xq[..., 1]
    pi = np.pi
    ue = np.stack([np.sin(pi * x) * np.cos(pi * y), -np.cos(pi * x) * np.sin(pi * y)], -1)
    pe = np.cos(pi * x) * np.cos(pi * y)
    _, _, eu, _ = problems.error_norms(level, u, p, ue, pe, 6)
    uq, pq = problems.evaluate_fields(level, u, p, 6)
    _, jxw = problems.q_points_real(level, 6)
    shift = np.sum((pq - pe) * jxw) / np.sum(jxw)  # the pressure is fixed up to a constant
    ep = np.sqrt(np.sum((pq - shift - pe) ** 2 * jxw))
    return eu, ep


def test_q3_manufactured_convergence_rates():
    errs = {}
    for degree in (2, 3):
        for n in (4, 8):
            levels, rhs = manufactured_problem(n, degree)
            o = Oracle(levels)
            f = levels[-1]
            o.set_viscosity(np.ones(f.n_cells), 0, 1.0)
            o.build_preconditioner(False)
            sol, info = o.solve(rhs, tol_rel=1e-12)
            assert info["status"] == 0
            errs[degree, n] = exact_errors(f, sol[: f.n_u], sol[f.n_u:])
    ru3 = errs[3, 4][0] / errs[3, 8][0]
    rp3 = errs[3, 4][1] / errs[3, 8][1]
    ru2 = errs[2, 4][0] / errs[2, 8][0]
    assert 13 < ru3 < 19, errs   # O(h^4)
    assert 6 < rp3 < 10, errs    # O(h^3)
    assert 6 < ru2 < 10, errs    # Q2: O(h^3)
    assert errs[3, 8][0] < 0.1 * errs[2, 8][0]
