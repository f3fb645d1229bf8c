"""Float-pair Gram-Schmidt of the GMRES / FGMRES Arnoldi steps
(gb_gmg_solve_params.orthogonalization = GB_GMG_GS_FLOAT_PAIR, the default)
against the FP64 passes (GB_GMG_GS_FP64) on the same handle: the same iteration
counts and solutions within 1e-10 relative (the passes differ in the last
~10 bits of each Hessenberg entry, far below the 1e-8 solver tolerance), for
FP64 and FP32 V-cycles, odd and even system sizes, short restarts (every
restart begins with an FP64 step that sets the scale of the next one), the
flexible and the non-flexible cheap solver and GMRES-IR; the float-pair
FP64-MG solve against the oracle's solve within 1e-8 with its FP64 residual
under the tolerance; and a restart cycle longer than 128 steps (FP64 passes
after the 128th basis vector)."""
import numpy as np
import pytest

from aspect_gb300 import gmg, problems
from oracle import Oracle
from tests.gpu_util import p_err, rel_err

pytestmark = pytest.mark.gpu

GS_FLOAT_PAIR, GS_FP64 = 0, 1


def _pair_solve(g, rhs, f, **kw):
    xa, oa = g.solve(rhs, orthogonalization=GS_FLOAT_PAIR, **kw)
    xb, ob = g.solve(rhs, orthogonalization=GS_FP64, **kw)
    assert oa["status"] == 0 and ob["status"] == 0
    assert oa["cheap_iterations"] == ob["cheap_iterations"], (oa, ob)
    assert oa["expensive_iterations"] == ob["expensive_iterations"], (oa, ob)
    assert rel_err(xa[: f.n_u], xb[: f.n_u]) < 1e-10
    assert p_err(xa[f.n_u:], xb[f.n_u:]) < 1e-10
    return xa, oa


@pytest.mark.parametrize("precision", [gmg.FP64, gmg.FP32])
@pytest.mark.parametrize("restart", [100, 7])
def test_float_pair_equals_fp64_passes_3d(precision, restart):
    P = problems.sinkers_3d(16, projection=1)
    g = gmg.from_problem(P)
    f = P.fine
    assert (f.n_u + f.n_p) % 2 == 0
    _pair_solve(g, P.rhs, f, linear_solver_tolerance=1e-8, mg_precision=precision, restart=restart)


def test_float_pair_odd_length_and_oracle():
    """2D SolCx (odd n_u + n_p: the last entry takes the kernels' scalar path):
    FP64-MG with the float-pair passes against the oracle's FP64 solve."""
    P = problems.solcx(6, density_sign=1.0)
    f = P.fine
    assert (f.n_u + f.n_p) % 2 == 1
    g = gmg.from_problem(P)
    x, out = _pair_solve(g, P.rhs, f, linear_solver_tolerance=1e-8, mg_precision=gmg.FP64, restart=9)
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    o.build_preconditioner(False)
    xr, info = o.solve(P.rhs, tol_rel=1e-8, restart=9)
    assert rel_err(x[: f.n_u], xr[: f.n_u]) < 1e-8
    assert p_err(x[f.n_u:], xr[f.n_u:]) < 1e-8
    assert abs(out["cheap_iterations"] - info["cheap_iterations"]) <= 1
    r = P.rhs - o.vmult(0, len(P.levels) - 1, x)
    assert np.linalg.norm(r) <= 1.01 * out["solver_tolerance"]


def test_float_pair_gmres_ir_and_nonflexible():
    P = problems.sinkers_3d(8)
    g = gmg.from_problem(P)
    f = P.fine
    _pair_solve(g, P.rhs, f, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32, krylov=gmg.GMRES_IR)
    # the expensive path (FGMRES with inner CG solves) after no cheap steps
    _pair_solve(g, P.rhs, f, linear_solver_tolerance=1e-6, mg_precision=gmg.FP64, n_cheap_steps=0)


def test_orthogonalization_value_is_checked():
    P = problems.sinkers_3d(4)
    g = gmg.from_problem(P)
    with pytest.raises(gmg.GmgError):
        g.solve(P.rhs, orthogonalization=2)


def test_float_pair_beyond_128_basis_vectors():
    """Spherical shell (about 190 iterations) with restart 200: the Arnoldi steps
    past 128 basis vectors run the FP64 passes inside a float-pair solve, the
    float-pair steps before them; the solution's FP64 residual, measured by the
    oracle, meets the tolerance and the iteration count matches the FP64
    passes' within one."""
    P = problems.spherical_shell(2)
    g = gmg.from_problem(P, options={"coarse_solver": gmg.COARSE_DENSE_FP64})
    xa, oa = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32, restart=200,
                     orthogonalization=GS_FLOAT_PAIR)
    xb, ob = g.solve(P.rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32, restart=200,
                     orthogonalization=GS_FP64)
    assert oa["status"] == 0 and ob["status"] == 0
    assert oa["cheap_iterations"] > 130, oa
    assert abs(oa["cheap_iterations"] - ob["cheap_iterations"]) <= 1, (oa, ob)
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    r = P.rhs - o.vmult(0, len(P.levels) - 1, xa)
    assert np.linalg.norm(r) <= 1.01 * oa["solver_tolerance"]
