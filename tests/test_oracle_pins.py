"""The CPU oracle against the reference's own regression outputs and against
brute-force assembled matrices. No GPU needed."""
import json
import os

import numpy as np
import pytest

from aspect_gb300 import fe, mesh, problems
from oracle import Oracle
from tests import numpy_reference as nr

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("nref", [2, 4])
def test_solcx_matches_reference_regression(nref):
    """sol_cx_2_gmg / sol_cx_4_gmg: iteration count and the four error norms."""
    golden = json.load(open(os.path.join(GOLDEN, "solcx_golden.json")))[str(2 ** nref)]
    exact = np.load(os.path.join(GOLDEN, "solcx_exact.npz"))
    P = problems.solcx(nref)
    f = P.fine
    assert (f.n_u, f.n_p) == (golden["n_u"], golden["n_p"])
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    o.build_preconditioner(False)
    x, info = o.solve(P.rhs, tol_rel=1e-7)
    assert info["status"] == 0
    assert info["cheap_iterations"] == golden["cheap_iterations"]
    assert info["expensive_iterations"] == golden["expensive_iterations"]
    u = x[: f.n_u].copy()
    p = x[f.n_u:] * P.pressure_scaling
    f.constraints_u.distribute(u)
    problems.normalize_pressure_surface(f, p)
    n = 2 ** nref
    errs = problems.error_norms(f, u, p, exact[f"u_{n}"], exact[f"p_{n}"])
    # the reference prints 7 significant digits
    np.testing.assert_allclose(errs, golden["errors"], rtol=2e-6)


def test_solcx_without_averaging_matches_reference_regression():
    """sol_cx_4_gmg_no_avg: no material averaging (per-point viscosity for the
    outer operators, the cellwise projection on every multigrid level, as the
    reference arranges it): the same 15 iterations and error norms as with
    averaging, since the viscosity jump lies on cell faces."""
    golden = json.load(open(os.path.join(GOLDEN, "solcx_golden.json")))["16_no_avg"]
    exact = np.load(os.path.join(GOLDEN, "solcx_exact.npz"))
    P = problems.solcx(4)
    f = P.fine
    xq, _ = problems.q_points_real(f)
    eta_q = np.where(xq[..., 0] < 0.5, 1.0, 1e6)
    o = Oracle(P.levels)
    o.set_viscosity(eta_q, 0, P.pressure_scaling, mg_finest_projected=True)
    o.build_preconditioner(False)
    x, info = o.solve(P.rhs, tol_rel=1e-7)
    assert info["status"] == 0 and info["cheap_iterations"] == golden["cheap_iterations"]
    u = x[: f.n_u].copy()
    p = x[f.n_u:] * P.pressure_scaling
    f.constraints_u.distribute(u)
    problems.normalize_pressure_surface(f, p)
    errs = problems.error_norms(f, u, p, exact["u_16"], exact["p_16"])
    np.testing.assert_allclose(errs, golden["errors"], rtol=2e-6)


def test_expensive_solver_matches_reference_regression():
    """no_cheap_gmg: SolCx 16x16 with no cheap steps (FGMRES with the expensive
    block preconditioner: CG on the velocity block to 1e-2 and on the Schur
    approximation to 1e-6, V-cycles as their preconditioners) and "harmonic
    average" of density as well as viscosity: 0+12 iterations and the four
    error norms the reference prints."""
    golden = json.load(open(os.path.join(GOLDEN, "solcx_golden.json")))["16_no_cheap"]
    exact = np.load(os.path.join(GOLDEN, "solcx_exact.npz"))
    P = problems.solcx(4, average_density=True)
    f = P.fine
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    o.build_preconditioner(False)
    x, info = o.solve(P.rhs, tol_rel=1e-7, n_cheap=0)
    assert info["status"] == 0
    assert (info["cheap_iterations"], info["expensive_iterations"]) == (golden["cheap_iterations"],
                                                                        golden["expensive_iterations"])
    u = x[: f.n_u].copy()
    p = x[f.n_u:] * P.pressure_scaling
    f.constraints_u.distribute(u)
    problems.normalize_pressure_surface(f, p)
    errs = problems.error_norms(f, u, p, exact["u_16"], exact["p_16"])
    np.testing.assert_allclose(errs, golden["errors"], rtol=2e-6)


def _small_problem(dim, n, per_q, seed=3):
    levels = mesh.box_hierarchy(dim, n)
    f = levels[-1]
    rng = np.random.default_rng(seed)
    nq = 3 ** dim
    eta = np.exp(rng.normal(size=(f.n_cells, nq) if per_q else f.n_cells))
    return levels, eta


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("per_q", [False, True])
def test_oracle_operators_match_assembled(dim, per_q):
    levels, eta = _small_problem(dim, 2, per_q)
    f = levels[-1]
    s = 3.7
    o = Oracle(levels)
    o.set_viscosity(eta, 0, s)
    eq = eta if per_q else np.repeat(eta[:, None], 3 ** dim, 1)
    A, BT, M = nr.stokes_blocks(f, eq, s)
    Cu = nr.constraint_matrix(f.n_u, f.constraints_u)
    mu = f.constraints_u.constrained_mask(f.n_u)
    Ac = nr.constrained_operator(A, Cu, Cu, mu)
    rng = np.random.default_rng(1)
    x = rng.normal(size=f.n_u + f.n_p)
    ya = o.vmult(1, len(levels) - 1, x[: f.n_u])
    np.testing.assert_allclose(ya, Ac @ x[: f.n_u], rtol=1e-12, atol=1e-12 * np.abs(ya).max())
    ym = o.vmult(3, len(levels) - 1, x[f.n_u:])
    np.testing.assert_allclose(ym, M @ x[f.n_u:], rtol=1e-12, atol=1e-12 * np.abs(ym).max())
    # full Stokes: [A BT; BT^T 0] with constrained velocity rows/cols
    BTc = Cu.T @ BT
    BTc[mu, :] = 0
    K = np.block([[Ac, BTc], [BTc.T, np.zeros((f.n_p, f.n_p))]])
    ys = o.vmult(0, len(levels) - 1, x)
    np.testing.assert_allclose(ys, K @ x, rtol=1e-12, atol=1e-12 * np.abs(ys).max())
    yb = o.vmult(2, len(levels) - 1, x[f.n_u:])
    np.testing.assert_allclose(yb, BTc @ x[f.n_u:], rtol=1e-12, atol=1e-12 * np.abs(yb).max())
    # diagonals
    o.build_preconditioner(False)
    dA = o.diagonal_inverse(len(levels) - 1, 0)
    ref = 1.0 / np.where(mu, 1.0, np.diag(Ac))
    np.testing.assert_allclose(dA, ref, rtol=1e-12)


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_transfer_is_exact_embedding(dim):
    """Prolongating a coarse FE function reproduces it at the fine DoF points."""
    levels = mesh.box_hierarchy(dim, 4, free_slip=False)
    o = Oracle(levels)
    c, f = levels[-2], levels[-1]

    def field(x, comp):
        return 1 + x[:, 0] ** 2 - 0.5 * x[:, 1] * (comp + 1) + (x[:, -1] ** 2 if dim == 3 else 0)

    uc = field(c.dof_points_u, c.dof_component_u)
    uf = o.transfer(len(levels) - 1, 0, False, uc)
    np.testing.assert_allclose(uf, field(f.dof_points_u, f.dof_component_u), rtol=1e-13, atol=1e-13)
    pc = 1 + c.dof_points_p.sum(1)
    pf = o.transfer(len(levels) - 1, 1, False, pc)
    np.testing.assert_allclose(pf, 1 + f.dof_points_p.sum(1), rtol=1e-13)
    # restriction is the transpose
    rng = np.random.default_rng(0)
    a, b = rng.normal(size=c.n_u), rng.normal(size=f.n_u)
    lhs = b @ o.transfer(len(levels) - 1, 0, False, a)
    rhs = a @ o.transfer(len(levels) - 1, 0, True, b)
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


@pytest.mark.parametrize("key,krylov", [("gmres", 0), ("idr2", 2)])
def test_nsinker_matches_reference_outputs(key, krylov):
    """The reference's NSinker benchmark on its 4^3 test mesh (3D, zero velocity on
    all faces, 4 sinkers, viscosity ratio 1e4, harmonic averaging of viscosity
    only, pressure scaling 1, tolerance 1e-6): the oracle prints the viscosity
    range, DoF counts, iteration counts and Schur-preconditioner applications of
    tests/nsinker_gmg_gc/screen-output (GMRES: 21, 22) and
    tests/nsinker_gmg_idr/screen-output (IDR(2): 9, 25)."""
    G = json.load(open(os.path.join(GOLDEN, "nsinker_golden.json")))
    ref = G[key]
    P = problems.nsinker(2, G["centres"], G["dynamic_viscosity_ratio"], G["sinker_density"], G["delta"],
                         G["omega"])
    f = P.fine
    assert (f.n_u, f.n_p) == (ref["n_u"], ref["n_p"])
    np.testing.assert_allclose([P.eta.min(), P.eta.max()], ref["viscosity_range"], rtol=5e-6)
    o = Oracle(P.levels)
    o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
    o.build_preconditioner(False)
    _, info = o.solve(P.rhs, tol_rel=G["linear_solver_tolerance"], n_cheap=G["n_cheap_steps"], n_expensive=0,
                      restart=G["restart"], krylov=krylov, idr_s=2)
    assert info["status"] == 0
    assert info["cheap_iterations"] == ref["cheap_iterations"]
    assert info["S_preconditioner_applications"] == ref["schur_applications"]


def test_nsinker_without_averaging_follows_reference_semantics():
    """tests/nsinker_gmg_no_avg (and nsinker_gmg_gc_no_avg): without averaging the
    reference keeps per-point viscosity for the outer operators but gives every
    multigrid level, the finest included, the cellwise (DGQ0) projection, so the
    V-cycle's finest level differs from the operator it preconditions: GMRES
    needs 172 iterations (174 Schur applications). The oracle with that
    arrangement (mg_finest_projected) lands within two iterations of it (a slow
    solve with two restarts amplifies last-digit differences of the projection).
    With the per-point table on the finest multigrid level as well (the
    library's GB_GMG_VISC_DGQ0 with per-point values) the V-cycle's finest level
    is the operator itself, and far fewer iterations reach the same 1e-6
    residual; the library's GB_GMG_VISC_NONE gives the reference's arrangement
    (GPU test in test_gpu_solve_parity.py)."""
    G = json.load(open(os.path.join(GOLDEN, "nsinker_golden.json")))
    ref = G["no_avg"]
    P = problems.nsinker(2, G["centres"], G["dynamic_viscosity_ratio"], G["sinker_density"], G["delta"],
                         G["omega"], averaging="none")
    np.testing.assert_allclose([P.eta.min(), P.eta.max()], ref["viscosity_range"], rtol=5e-6)
    its = {}
    for flag in (True, False):
        o = Oracle(P.levels)
        o.set_viscosity(P.eta, P.projection, P.pressure_scaling, mg_finest_projected=flag)
        o.build_preconditioner(False)
        _, info = o.solve(P.rhs, tol_rel=G["linear_solver_tolerance"], n_cheap=G["n_cheap_steps"], n_expensive=0,
                          restart=G["restart"])
        assert info["status"] == 0
        its[flag] = info["cheap_iterations"]
    assert abs(its[True] - ref["cheap_iterations"]) <= 2, its
    assert its[False] < ref["cheap_iterations"] // 2, its


@pytest.mark.parametrize("dim", [2, 3])
def test_oracle_geometry_table_matches_q2_mapping(dim):
    """GEOM_TABLE (the caller's inverse Jacobians and |det J| per Gauss point)
    built from a level's Q2 mapping gives the same operators as GEOM_Q2."""
    base = mesh.box_hierarchy(dim, 4)
    q2 = [mesh.to_q2_geometry(l, mesh.smooth_distortion(0.05)) for l in base]
    tab = [mesh.to_table_geometry(l) for l in q2]
    eta = np.exp(np.random.default_rng(3).uniform(-1, 1, size=(base[-1].n_cells, 3 ** dim)))
    oa, ob = Oracle(q2), Oracle(tab)
    oa.set_viscosity(eta, 0, 1.3, 1)
    ob.set_viscosity(eta, 0, 1.3, 1)
    top = len(base) - 1
    m = q2[-1]
    x = np.random.default_rng(4).normal(size=m.n_u + m.n_p)
    for op, src in ((0, x), (1, x[: m.n_u]), (2, x[m.n_u:]), (3, x[m.n_u:])):
        a, b = oa.vmult(op, top, src), ob.vmult(op, top, src)
        assert np.linalg.norm(a - b) <= 1e-13 * np.linalg.norm(a), op
