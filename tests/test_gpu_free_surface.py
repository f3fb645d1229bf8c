"""Free-surface stabilisation faces on the GPU (gb_gmg_set_free_surface) against
the oracle (whose face term is checked against the dense face matrix and closed-
form surface integrals in test_free_surface_cpu.py): the outer Stokes operator
on lattice, indexed, distorted-Q2, hanging-node, curved-shell and geometry-table
levels, with the library's own face normals (box and Q2 geometry) against the
harness's, FP64 within 1e-12 and FP32 within 2e-5; together with Newton terms;
correct_stokes_rhs with the face term (the reference's :709-746) against the
dense form; and a solve with the face term whose FP64 residual the oracle checks.
The multigrid levels carry no face term (as in the reference)."""
import numpy as np
import pytest

from aspect_gb300 import gmg, mesh, octree, shell
from oracle import Oracle
from tests import numpy_reference as nr
from tests.gpu_util import random_eta, rel_err

pytestmark = pytest.mark.gpu


def _levels(case):
    if case in ("box3d", "box3d-indexed"):
        return mesh.box_hierarchy(3, 4, open_faces=(5,))
    if case == "box2d":
        return mesh.box_hierarchy(2, 8, open_faces=(3,))
    if case == "q2-distorted2d":
        return [mesh.to_q2_geometry(l, mesh.smooth_distortion()) for l in mesh.box_hierarchy(2, 8, open_faces=(3,))]
    if case == "table3d":
        return [mesh.to_table_geometry(mesh.to_q2_geometry(l, mesh.smooth_distortion()))
                for l in mesh.box_hierarchy(3, 4, open_faces=(5,))]
    if case == "adaptive2d":
        leaves = octree.sphere_refined_leaves(2, 3, 1, (0.5, 0.9), 0.2)
        return octree.hierarchy(leaves, 2, free_slip=False)  # hanging nodes on the open top
    return shell.hierarchy(1, 3, 0.55, 1.0)


def _faces(case, level):
    if case == "shell":
        return mesh.boundary_faces(level, lambda x: np.abs(np.linalg.norm(x, axis=1) - 1.0) < 1e-9)
    d = level.dim - 1
    return mesh.boundary_faces(level, lambda x: np.abs(x[:, d] - 1.0) < 1e-9)


def _geometry_source(case, level):
    """The level whose mapping the harness evaluates: a geometry-table level
    carries no mapping, so its faces come from the Q2 level it was tabulated from."""
    if case != "table3d":
        return level
    return mesh.to_q2_geometry(mesh.box_hierarchy(3, 4, open_faces=(5,))[-1], mesh.smooth_distortion())


def _setup(case, seed=3):
    levels = _levels(case)
    f = levels[-1]
    fc, fn = _faces(case, _geometry_source(case, f))
    assert len(fc) > 0
    rng = np.random.default_rng(seed)
    T = rng.normal(size=(len(fc), 3 ** (f.dim - 1), f.dim))
    return levels, f, fc, fn, T


@pytest.mark.parametrize("case", ["box3d", "box3d-indexed", "box2d", "q2-distorted2d", "table3d", "adaptive2d",
                                  "shell"])
def test_free_surface_operator_matches_oracle(case):
    levels, f, fc, fn, T = _setup(case)
    eta = random_eta(f, True, seed=5)
    g = gmg.StokesMatrixFreeGPU(f.dim, len(levels), {"force_indexed_layout": int(case == "box3d-indexed")})
    g.setup_dofs(levels)
    g.assemble(eta, 0, 1.3)
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 1.3)
    # the oracle takes the harness's normals; the library computes its own
    # except on a geometry-table level, which needs the caller's
    nj = mesh.face_normal_jxw(_geometry_source(case, f), fc, fn)
    g.set_free_surface(fc, fn, T, nj if case == "table3d" else None)
    o.set_free_surface(fc, fn, T, nj)
    top = len(levels) - 1
    x = np.random.default_rng(1).normal(size=f.n_u + f.n_p)
    y = o.vmult(0, top, x)
    assert rel_err(g.vmult(gmg.OP_STOKES, top, x, gmg.FP64), y) < 1e-12
    assert rel_err(g.vmult(gmg.OP_STOKES, top, x, gmg.FP32), y) < 2e-5
    # the face term is present (and the A block / levels do not carry it)
    o.set_free_surface()
    y0 = o.vmult(0, top, x)
    assert rel_err(y, y0) > 1e-6
    assert rel_err(g.vmult(gmg.OP_A, top, x[: f.n_u], gmg.FP64), o.vmult(1, top, x[: f.n_u])) < 1e-12
    g.set_free_surface()
    assert rel_err(g.vmult(gmg.OP_STOKES, top, x, gmg.FP64), y0) < 1e-12


def test_free_surface_with_newton_terms():
    levels, f, fc, fn, T = _setup("box3d")
    eta = random_eta(f, True, seed=2)
    g = gmg.StokesMatrixFreeGPU(3, len(levels))
    g.setup_dofs(levels)
    g.assemble(eta, 0, 1.0)
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 1.0)
    rng = np.random.default_rng(9)
    E = 0.5 * rng.normal(size=(f.n_cells, 27, 6))
    t = dict(newton=True, symmetrize=True, strain_rate=E, d_eta_d_strain_rate=0.3 * E,
             d_eta_d_pressure=0.1 * rng.normal(size=(f.n_cells, 27)))
    g.set_newton_terms(**t)
    o.set_newton_terms(**t)
    g.set_free_surface(fc, fn, T)
    o.set_free_surface(fc, fn, T)
    x = rng.normal(size=f.n_u + f.n_p)
    y = o.vmult(0, len(levels) - 1, x)
    assert rel_err(g.vmult(gmg.OP_STOKES, len(levels) - 1, x, gmg.FP64), y) < 1e-12
    assert rel_err(g.vmult(gmg.OP_STOKES, len(levels) - 1, x, gmg.FP32), y) < 2e-5


@pytest.mark.parametrize("case", ["box3d", "adaptive2d"])
def test_correct_stokes_rhs_with_free_surface(case):
    levels, f, fc, fn, T = _setup(case, seed=4)
    eta = random_eta(f, True)
    g = gmg.StokesMatrixFreeGPU(f.dim, len(levels))
    g.setup_dofs(levels)
    g.assemble(eta, 0, 1.7)
    g.set_free_surface(fc, fn, T)
    rng = np.random.default_rng(11)
    mu = f.constraints_u.constrained_mask(f.n_u)
    u0 = np.zeros(f.n_u + f.n_p)
    u0[: f.n_u][mu] = rng.normal(size=mu.sum())
    rhs = rng.normal(size=f.n_u + f.n_p)
    got = g.correct_stokes_rhs(u0, rhs)
    A, BT, M = nr.stokes_blocks(f, eta, 1.7)
    A = A + nr.free_surface_matrix(f, fc, fn, T, mesh.face_normal_jxw(f, fc, fn))
    K = np.block([[A, BT], [BT.T, np.zeros((f.n_p, f.n_p))]])
    C = np.zeros((f.n_u + f.n_p, f.n_u + f.n_p))
    C[: f.n_u, : f.n_u] = nr.constraint_matrix(f.n_u, f.constraints_u)
    C[f.n_u:, f.n_u:] = nr.constraint_matrix(f.n_p, f.constraints_p)
    corr = C.T @ (K @ u0)
    assert rel_err(got - rhs, -corr) < 1e-12
    assert np.array_equal(got[: f.n_u][mu], rhs[: f.n_u][mu])


def test_solve_with_free_surface():
    """An open-top box with the stabilisation T = rho dt theta |g| g_hat (g = -z):
    the solve meets its tolerance on the operator with the face term, which the
    oracle's FP64 product confirms."""
    levels = mesh.box_hierarchy(3, 8, open_faces=(5,))
    f = levels[-1]
    fc, fn = _faces("box3d", f)
    T = np.zeros((len(fc), 9, 3))
    T[..., 2] = -0.5 * 1.0 * 0.8  # rho dt theta |g| g_hat
    eta = random_eta(f, False, seed=6, contrast=1.0)
    g = gmg.StokesMatrixFreeGPU(3, len(levels))
    g.setup_dofs(levels)
    g.assemble(eta, 0, 1.0)
    g.set_free_surface(fc, fn, T)
    g.build_preconditioner()
    rng = np.random.default_rng(2)
    rhs = np.concatenate([rng.normal(size=f.n_u), np.zeros(f.n_p)])
    rhs[f.constraints_u.rows] = 0.0
    x, out = g.solve(rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    assert out["status"] == 0
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 1.0)
    o.set_free_surface(fc, fn, T)
    r = np.linalg.norm(rhs - o.vmult(0, len(levels) - 1, x))
    assert r <= 1.01 * out["solver_tolerance"], (r, out)


def test_free_surface_argument_checks():
    levels, f, fc, fn, T = _setup("box3d")
    g = gmg.StokesMatrixFreeGPU(3, len(levels))
    g.setup_dofs(levels)
    with pytest.raises(gmg.GmgError):
        g.set_free_surface(np.r_[fc, fc[:1]], np.r_[fn, fn[:1]], np.concatenate([T, T[:1]]))  # a face twice
    with pytest.raises(gmg.GmgError):
        g.set_free_surface(fc, np.full_like(fn, 6), T)  # face number out of range
    with pytest.raises(gmg.GmgError):
        g.set_free_surface(fc + f.n_cells, fn, T)  # cell out of range
    bad = T.copy()
    bad[0, 0, 0] = np.nan
    with pytest.raises(gmg.GmgError):
        g.set_free_surface(fc, fn, bad)
    tl = _levels("table3d")
    h = gmg.StokesMatrixFreeGPU(3, len(tl))
    h.setup_dofs(tl)
    with pytest.raises(gmg.GmgError):
        h.set_free_surface(fc, fn, T)  # a geometry-table level needs normal_jxw
