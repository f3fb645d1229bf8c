"""Spherical-shell meshes (curved Q2 cells, no-normal-flux lines that couple
velocity components) checked on the CPU: the oracle against assembled matrices,
and the rigid rotations as exact null vectors of the constrained A block."""
import numpy as np

from aspect_gb300 import problems, shell
from oracle import Oracle
from tests import numpy_reference as nr


def test_shell_mesh_counts():
    levels = shell.hierarchy(1)
    assert [l.n_cells for l in levels] == [96, 768]
    f = levels[-1]
    assert f.constraints_u.n_lines == len(np.unique(f.constraints_u.rows))
    r = np.linalg.norm(f.q2_support_points(), axis=-1)
    assert r.min() > 0.55 - 1e-12 and r.max() < 1.0 + 1e-12


def test_shell_operators_match_assembled_and_rotations_are_null():
    levels = shell.hierarchy(0)
    f = levels[-1]
    rng = np.random.default_rng(3)
    eta = np.exp(rng.uniform(-1, 1, size=(f.n_cells, 27)))
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 2.0)
    A, BT, M = nr.stokes_blocks(f, eta, 2.0)
    Cu = nr.constraint_matrix(f.n_u, f.constraints_u)
    mu = f.constraints_u.constrained_mask(f.n_u)
    Ac = nr.constrained_operator(A, Cu, Cu, mu)
    x = rng.normal(size=f.n_u)
    y = o.vmult(1, 0, x)
    assert np.linalg.norm(y - Ac @ x) <= 1e-12 * np.linalg.norm(y)
    for mode in shell.rotation_modes(f):
        mode[mu] = 0.0  # constrained entries are implied by their lines
        ya = o.vmult(1, 0, mode)
        assert np.linalg.norm(ya) <= 1e-10 * np.linalg.norm(o.vmult(1, 0, x)) * np.linalg.norm(mode) / np.linalg.norm(x)


def test_shell_problem_oracle_solve():
    P = problems.spherical_shell(1)
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    o.build_preconditioner(False)
    x, info = o.solve(P.rhs, tol_rel=1e-8)
    assert info["status"] == 0
    assert np.linalg.norm(P.rhs - o.vmult(0, 1, x)) <= 1.01 * info["solver_tolerance"]


def _adaptive_cells(n_ref, seed=4):
    cells = shell.all_cells(4, n_ref)
    ind = np.random.default_rng(seed).uniform(size=len(cells))
    return shell.refine_fixed_fraction(cells, ind, 0.3)


def test_adaptive_shell_hanging_lines():
    """Without free slip every line is a hanging-node line: masters are
    unconstrained, weights sum to one (constants are reproduced), and the
    interpolated position of a Q2 hanging node differs from its position on the
    sphere by the Q2 geometry error of the coarse face, which falls like h^3."""
    mismatch = []
    for n_ref in (0, 1):
        leaves = _adaptive_cells(n_ref)
        assert {c[1] for c in leaves} == {n_ref, n_ref + 1}
        f = shell.adaptive_hierarchy(leaves, free_slip=False)[-1]
        for cons, n, pts in ((f.constraints_u, f.n_u, f.dof_points_u), (f.constraints_p, f.n_p, f.dof_points_p)):
            assert cons.n_lines > 0
            mask = cons.constrained_mask(n)
            assert not mask[cons.cols].any()
            sums = np.add.reduceat(cons.weights, cons.ptr[:-1])
            assert np.allclose(sums, 1.0, atol=1e-13)
            if cons is f.constraints_u:
                interp = np.stack([np.add.reduceat(cons.weights * pts[cons.cols, e], cons.ptr[:-1])
                                   for e in range(3)], -1)
                mismatch.append(np.abs(interp - pts[cons.rows]).max())
    assert mismatch[1] < 1e-2 and mismatch[0] / mismatch[1] > 6, mismatch


def test_adaptive_shell_fixed_fraction_marks_largest_indicators():
    cells = shell.all_cells(4, 0)
    ind = np.arange(len(cells), dtype=float)
    out = shell.refine_fixed_fraction(cells, ind, 0.3)
    refined = {c[2:] + (c[0],) for c in cells} - {c[2:] + (c[0],) for c in out if c[1] == 0}
    n_ref = len(cells) - sum(1 for c in out if c[1] == 0)
    top = np.sort(ind)[::-1]
    assert top[:n_ref - 1].sum() < 0.3 * ind.sum() <= top[:n_ref].sum()
    assert len(refined) == n_ref and len(out) == len(cells) + 7 * n_ref


def test_adaptive_shell_operators_match_assembled():
    levels = shell.adaptive_hierarchy(_adaptive_cells(0))
    f = levels[-1]
    assert f.constraints_u.n_lines > 0 and f.constraints_p.n_lines > 0
    rng = np.random.default_rng(8)
    eta = np.exp(rng.uniform(-1, 1, size=(f.n_cells, 27)))
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 2.0)
    A, BT, M = nr.stokes_blocks(f, eta, 2.0)
    top = len(levels) - 1
    for op, K, cons, n in ((1, A, f.constraints_u, f.n_u), (3, M, f.constraints_p, f.n_p)):
        C = nr.constraint_matrix(n, cons)
        Kc = nr.constrained_operator(K, C, C, cons.constrained_mask(n))
        x = rng.normal(size=n)
        y = o.vmult(op, top, x)
        assert np.linalg.norm(y - Kc @ x) <= 1e-12 * np.linalg.norm(y)
