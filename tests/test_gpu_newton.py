"""Newton-derivative and prescribed-dilation terms of the outer Stokes operator
on the GPU (gb_gmg_set_newton_terms) against the oracle (whose Newton operator
is checked against the derivative of the nonlinear residual in
test_newton_cpu.py): every flag combination of OperatorCellData
(matrix_free_operators.cc:400-538), 2D and 3D, lattice and indexed levels,
FP64 within 1e-12 and FP32 within 2e-5; a Newton-update solve
(solve_newton_system) meets its tolerance on the Newton operator."""
import itertools

import numpy as np
import pytest

from aspect_gb300 import gmg
from oracle import Oracle
from tests.gpu_util import hierarchy, random_eta, rel_err

pytestmark = pytest.mark.gpu


def _tables(f, seed):
    rng = np.random.default_rng(seed)
    nq = 3 ** f.dim
    ns = 6 if f.dim == 3 else 3
    E = 0.5 * rng.normal(size=(f.n_cells, nq, ns))
    return dict(strain_rate=E, d_eta_d_strain_rate=0.3 * E + 0.1 * rng.normal(size=E.shape),
                d_eta_d_pressure=0.2 * rng.normal(size=(f.n_cells, nq)),
                dilation_lhs=0.1 * rng.normal(size=(f.n_cells, nq)),
                d_dilation_d_strain_rate=0.1 * rng.normal(size=(f.n_cells, nq, ns)),
                d_dilation_d_pressure=0.1 * rng.normal(size=(f.n_cells, nq)))


FLAGS = [dict(newton=n, symmetrize=s, average=a, dilation=d)
         for n, s, a, d in itertools.product([True], [False, True], [False, True], [False, True])]
FLAGS.append(dict(newton=False, symmetrize=False, average=False, dilation=True))


@pytest.mark.parametrize("dim,n,geometry,compressible", [(3, 4, "box", 0), (2, 8, "q2-distorted", 1),
                                                         (3, 4, "box", 1)])
def test_newton_stokes_operator_matches_oracle(dim, n, geometry, compressible):
    levels = hierarchy(dim, n, geometry)
    f = levels[-1]
    eta = random_eta(f, True, seed=3)
    s = 1.7
    g = gmg.StokesMatrixFreeGPU(dim, len(levels))
    g.setup_dofs(levels)
    g.assemble(eta, 0, s, compressible)
    o = Oracle(levels)
    o.set_viscosity(eta, 0, s, compressible)
    t = _tables(f, dim + compressible)
    top = len(levels) - 1
    x = np.random.default_rng(1).normal(size=f.n_u + f.n_p)
    for flags in FLAGS:
        g.set_newton_terms(**flags, **t)
        o.set_newton_terms(**flags, **t)
        y = o.vmult(0, top, x)
        assert rel_err(g.vmult(gmg.OP_STOKES, top, x, gmg.FP64), y) < 1e-12, flags
        assert rel_err(g.vmult(gmg.OP_STOKES, top, x, gmg.FP32), y) < 2e-5, flags
    g.set_newton_terms()  # cleared: the plain operator again
    o.set_newton_terms()
    assert rel_err(g.vmult(gmg.OP_STOKES, top, x, gmg.FP64), o.vmult(0, top, x)) < 1e-12


def test_newton_update_solve():
    """solve_newton_system: zero initial guess, tolerance rel_tol |rhs|; the FGMRES
    product carries the Newton terms (symmetrised, as the reference's default
    stabilisation gives), the V-cycles the Picard levels."""
    levels = hierarchy(3, 8, "box")
    f = levels[-1]
    eta = random_eta(f, True, seed=4, contrast=1.0)
    g = gmg.StokesMatrixFreeGPU(3, len(levels))
    g.setup_dofs(levels)
    g.assemble(eta, 0, 1.0)
    t = _tables(f, 7)
    t["d_eta_d_strain_rate"] = 0.05 * t["strain_rate"]
    g.set_newton_terms(newton=True, symmetrize=True, **{k: t[k] for k in
                       ("strain_rate", "d_eta_d_strain_rate", "d_eta_d_pressure")})
    g.build_preconditioner()
    rhs = np.concatenate([np.random.default_rng(2).normal(size=f.n_u), np.zeros(f.n_p)])
    rhs[f.constraints_u.rows] = 0.0
    x0 = np.full(f.n_u + f.n_p, 7.0)  # ignored: a Newton update starts from zero
    x, out = g.solve(rhs, x0=x0, linear_solver_tolerance=1e-8, solve_newton_system=1, mg_precision=gmg.FP32)
    assert out["status"] == 0
    assert abs(out["initial_nonlinear_residual"] - np.linalg.norm(rhs)) <= 1e-12 * np.linalg.norm(rhs)
    assert abs(out["solver_tolerance"] - 1e-8 * np.linalg.norm(rhs)) <= 1e-20 + 1e-12 * out["solver_tolerance"]
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 1.0)
    o.set_newton_terms(newton=True, symmetrize=True, **{k: t[k] for k in
                       ("strain_rate", "d_eta_d_strain_rate", "d_eta_d_pressure")})
    r = np.linalg.norm(rhs - o.vmult(0, len(levels) - 1, x))
    assert r <= 1.01 * out["solver_tolerance"], (r, out)
