"""Adaptive meshes with hanging nodes (the caller-side stand-in for deal.II's
hanging-node constraints), checked without a GPU: conformity of the closed
constraints, the oracle's constrained operators against assembled matrices,
and exact transfers across the capped-depth hierarchy."""
import numpy as np
import pytest

from aspect_gb300 import octree
from oracle import Oracle
from tests import numpy_reference as nr


def _levels(dim, base, nad, free_slip=True):
    leaves = octree.sphere_refined_leaves(dim, base, nad, (0.5,) * dim, 0.2 if dim == 3 else 0.3)
    return octree.hierarchy(leaves, dim, free_slip)


@pytest.mark.parametrize("dim,base,nad", [(2, 2, 2), (3, 2, 1)])
def test_hanging_constraints_reproduce_quadratic_fields(dim, base, nad):
    f = _levels(dim, base, nad, free_slip=False)[-1]
    assert f.constraints_u.n_lines > 0 and f.constraints_p.n_lines > 0
    x = f.dof_points_u
    c = f.dof_component_u
    exact = 1 + x[:, 0] ** 2 - 0.7 * x[:, 1] * x[:, -1] + 0.3 * c + x[:, 0] * x[:, 1]
    u = exact.copy()
    u[f.constraints_u.rows] = 12345.0
    f.constraints_u.distribute(u)
    np.testing.assert_allclose(u, exact, atol=1e-13)
    xp = f.dof_points_p
    pe = 1 + 2 * xp[:, 0] - xp[:, -1]
    p = pe.copy()
    p[f.constraints_p.rows] = -1.0
    f.constraints_p.distribute(p)
    np.testing.assert_allclose(p, pe, atol=1e-13)


@pytest.mark.parametrize("dim,base,nad", [(2, 2, 2), (3, 1, 1)])
def test_oracle_operators_on_adaptive_mesh_match_assembled(dim, base, nad):
    levels = _levels(dim, base, nad)
    f = levels[-1]
    rng = np.random.default_rng(4)
    eta = np.exp(rng.uniform(-1, 1, size=(f.n_cells, 3 ** dim)))
    s = 1.7
    o = Oracle(levels)
    o.set_viscosity(eta, 0, s)
    A, BT, M = nr.stokes_blocks(f, eta, s)
    Cu = nr.constraint_matrix(f.n_u, f.constraints_u)
    Cp = nr.constraint_matrix(f.n_p, f.constraints_p)
    mu = f.constraints_u.constrained_mask(f.n_u)
    mp = f.constraints_p.constrained_mask(f.n_p)
    Ac = nr.constrained_operator(A, Cu, Cu, mu)
    Mc = nr.constrained_operator(M, Cp, Cp, mp)
    xu, xp = rng.normal(size=f.n_u), rng.normal(size=f.n_p)
    top = len(levels) - 1
    ya = o.vmult(1, top, xu)
    assert np.linalg.norm(ya - Ac @ xu) <= 1e-12 * np.linalg.norm(ya)
    ym = o.vmult(3, top, xp)
    assert np.linalg.norm(ym - Mc @ xp) <= 1e-12 * np.linalg.norm(ym)
    BTc = Cu.T @ BT @ Cp
    BTc[mu, :] = 0
    BTc[:, mp] = 0
    yb = o.vmult(2, top, xp)
    assert np.linalg.norm(yb - BTc @ xp) <= 1e-12 * np.linalg.norm(yb)
    assert np.allclose(Ac, Ac.T, atol=1e-12 * np.abs(Ac).max())


@pytest.mark.parametrize("dim,base,nad", [(2, 2, 2), (3, 2, 1)])
def test_transfers_are_exact_across_hanging_nodes(dim, base, nad):
    levels = _levels(dim, base, nad, free_slip=False)
    o = Oracle(levels)
    for l in range(1, len(levels)):
        c, f = levels[l - 1], levels[l]

        def field(x, comp):
            return 1 + x[:, 0] ** 2 - 0.5 * x[:, 1] * (comp + 1) + x[:, -1] * x[:, 0]

        uc = field(c.dof_points_u, c.dof_component_u)
        uf = o.transfer(l, 0, False, uc)
        ref = field(f.dof_points_u, f.dof_component_u)
        free = ~f.constraints_u.constrained_mask(f.n_u)
        np.testing.assert_allclose(uf[free], ref[free], atol=1e-12)
        pc = 1 + c.dof_points_p.sum(1)
        pf = o.transfer(l, 1, False, pc)
        freep = ~f.constraints_p.constrained_mask(f.n_p)
        np.testing.assert_allclose(pf[freep], (1 + f.dof_points_p.sum(1))[freep], atol=1e-12)
