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
