"""GPU path (libgb_gmg.so through the C ABI) against the CPU oracle on the same
seeded inputs. Tolerances: FP64 operator results within 1e-12 relative (2-norm),
FP32 level operators within 2e-6 relative, FP32 V-cycles within 1e-4."""
import numpy as np
import pytest

from aspect_gb300 import gmg, mesh, problems
from oracle import Oracle
from tests.gpu_util import hierarchy, random_eta, rel_err

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 2e-6

CASES = [
    # dim, n, geometry, permute, per_q, compressible, force_indexed
    (2, 8, "box", False, False, 0, 0),
    (2, 8, "box", True, True, 1, 0),
    (2, 8, "q2-distorted", False, True, 0, 0),
    (3, 4, "box", False, False, 0, 0),
    (3, 8, "box", False, True, 0, 0),
    (3, 4, "box", True, True, 1, 0),
    (3, 4, "box", False, True, 0, 1),
    (3, 4, "q2-distorted", False, True, 0, 0),
]


def _pair(case):
    dim, n, geom, perm, per_q, comp, force = case
    levels = hierarchy(dim, n, geom, perm)
    eta = random_eta(levels[-1], per_q)
    s = 2.5
    g = gmg.StokesMatrixFreeGPU(dim, len(levels), {"force_indexed_layout": force})
    g.setup_dofs(levels)
    g.assemble(eta, 0, s, comp)
    o = Oracle(levels)
    o.set_viscosity(eta, 0, s, comp)
    return levels, g, o


@pytest.fixture(scope="module", params=CASES, ids=lambda c: "-".join(map(str, c)))
def pair(request):
    return _pair(request.param)


def test_vmult_all_operators_all_levels(pair):
    levels, g, o = pair
    rng = np.random.default_rng(7)
    for lev, m in enumerate(levels):
        for op in range(4):
            n_in = m.n_u + m.n_p if op == 0 else (m.n_u if op == 1 else m.n_p)
            x = rng.normal(size=n_in)
            y_ref = o.vmult(op, lev, x)
            y64 = g.vmult(op, lev, x, gmg.FP64)
            assert rel_err(y64, y_ref) < TOL64, (lev, op, rel_err(y64, y_ref))
            y32 = g.vmult(op, lev, x, gmg.FP32)
            assert rel_err(y32, y_ref) < TOL32 * 10, (lev, op, rel_err(y32, y_ref))


def test_diagonals_and_transfers(pair):
    levels, g, o = pair
    g.build_preconditioner()
    o.build_preconditioner(False)
    for lev, m in enumerate(levels):
        for block in (0, 1):
            d_ref = o.diagonal_inverse(lev, block)
            assert rel_err(g.diagonal_inverse(lev, block, gmg.FP64), d_ref) < TOL64
            assert rel_err(g.diagonal_inverse(lev, block, gmg.FP32), d_ref) < TOL32 * 10
    rng = np.random.default_rng(3)
    for lev in range(1, len(levels)):
        for block in (0, 1):
            c, f = levels[lev - 1], levels[lev]
            xc = rng.normal(size=c.n_u if block == 0 else c.n_p)
            xf = rng.normal(size=f.n_u if block == 0 else f.n_p)
            assert rel_err(g.transfer(lev, block, False, xc), o.transfer(lev, block, False, xc)) < 1e-13
            assert rel_err(g.transfer(lev, block, True, xf), o.transfer(lev, block, True, xf)) < 1e-13
            assert rel_err(g.transfer(lev, block, True, xf, gmg.FP32), o.transfer(lev, block, True, xf)) < 1e-6


def test_eigenvalues_and_vcycles(pair):
    levels, g, o = pair
    g.build_preconditioner()
    o.build_preconditioner(False)
    o.estimate_eigenvalues()
    for lev in range(len(levels)):
        for block in (0, 1):
            e_ref = o.eigenvalues(lev, block)
            e64 = g.eigenvalues(lev, block, gmg.FP64)
            assert abs(e64[1] - e_ref[1]) < 1e-8 * abs(e_ref[1]), (lev, block, e64, e_ref)
            e32 = g.eigenvalues(lev, block, gmg.FP32)
            assert abs(e32[1] - e_ref[1]) < 1e-3 * abs(e_ref[1]), (lev, block, e32, e_ref)
            # use the GPU's FP64 estimates in the oracle so the V-cycles are comparable
            o.set_eigenvalues(lev, block, e64)
    rng = np.random.default_rng(11)
    f = levels[-1]
    for block in (0, 1):
        r = rng.normal(size=f.n_u if block == 0 else f.n_p)
        v_ref = o.vcycle(block, r)
        assert rel_err(g.vcycle(block, r, gmg.FP64), v_ref) < 1e-10
    r = rng.normal(size=f.n_u + f.n_p)
    b_ref = o.block_preconditioner(r)
    assert rel_err(g.block_preconditioner(r, gmg.FP64), b_ref) < 1e-10
    # FP32 V-cycle against the FP64 one with the same smoother intervals
    for lev in range(len(levels)):
        for block in (0, 1):
            g.set_eigenvalues(lev, block, gmg.FP32, g.eigenvalues(lev, block, gmg.FP64))
    for block in (0, 1):
        r = rng.normal(size=f.n_u if block == 0 else f.n_p)
        assert rel_err(g.vcycle(block, r, gmg.FP32), g.vcycle(block, r, gmg.FP64)) < 1e-5


def test_adjoint_gradient_matches_cpu_adjoint(pair):
    levels, g, o = pair
    f = levels[-1]
    rng = np.random.default_rng(5)
    u, lam = rng.normal(size=f.n_u), rng.normal(size=f.n_u)
    assert rel_err(g.adjoint_gradient(u, lam), o.adjoint_gradient(u, lam)) < TOL64


def test_fp32_vcycles_with_fused_mass_levels():
    """16^3 sinkers: the FP32 mass V-cycle runs levels 0-3 (<= 729 pressure nodes)
    in one single-block launch and level 4 with per-step launches; the FP32
    block preconditioner also forms B^T p in FP32. Both stay within FP32 rounding
    of the FP64 path when the smoother intervals are the same."""
    P = problems.sinkers_3d(16)
    g = gmg.from_problem(P)
    for lev in range(len(P.levels)):
        for block in (0, 1):
            g.set_eigenvalues(lev, block, gmg.FP32, g.eigenvalues(lev, block, gmg.FP64))
    rng = np.random.default_rng(21)
    f = P.fine
    rp = rng.normal(size=f.n_p)
    assert rel_err(g.vcycle(1, rp, gmg.FP32), g.vcycle(1, rp, gmg.FP64)) < 1e-5
    r = rng.normal(size=f.n_u + f.n_p)
    assert rel_err(g.block_preconditioner(r, gmg.FP32), g.block_preconditioner(r, gmg.FP64)) < 1e-5


def test_vmult_is_bit_reproducible():
    levels, g, o = _pair((3, 8, "box", False, True, 0, 0))
    x = np.random.default_rng(0).normal(size=levels[-1].n_u + levels[-1].n_p)
    a = g.vmult(0, len(levels) - 1, x)
    b = g.vmult(0, len(levels) - 1, x)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("per_q,comp", [(False, 0), (True, 0), (True, 1)])
def test_fp32_a_block_on_large_lattice_level(per_q, comp):
    """16^3 box (4,096 cells on the finest level, above the small-level kernel's
    512): the FP32 A-block cell pass of large lattice levels against the oracle,
    with cellwise and per-point viscosity, incompressible and compressible, and
    the free-slip constraints of all six walls."""
    levels = hierarchy(3, 16)
    eta = random_eta(levels[-1], per_q)
    g = gmg.StokesMatrixFreeGPU(3, len(levels))
    g.setup_dofs(levels)
    g.assemble(eta, 0, 2.5, comp)
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 2.5, comp)
    rng = np.random.default_rng(31)
    top = len(levels) - 1
    for _ in range(2):
        x = rng.normal(size=levels[-1].n_u)
        y_ref = o.vmult(1, top, x)
        assert rel_err(g.vmult(1, top, x, gmg.FP32), y_ref) < TOL32 * 10
        assert rel_err(g.vmult(1, top, x, gmg.FP64), y_ref) < TOL64


@pytest.mark.parametrize("n,per_q", [(16, True), (32, True), (32, False)])
def test_fused_ablock_operator(n, per_q):
    """The fused FP32 A-block operator of large lattice levels (one cell-and-gather
    pass per tile of 16 x 8 cells and a face pass) against the two-pass operator
    and the oracle, on every level where it applies; its Chebyshev and residual
    epilogues through a V-cycle and a mixed solve; bit-reproducibility."""
    levels = mesh.box_hierarchy(3, n)
    f = levels[-1]
    eta = random_eta(f, per_q, seed=n)
    fused = gmg.StokesMatrixFreeGPU(3, len(levels), {"fused_a_min_cells": 1})
    plain = gmg.StokesMatrixFreeGPU(3, len(levels), {"fused_a_min_cells": 0})
    for g in (fused, plain):
        g.setup_dofs(levels)
        g.assemble(eta, 0, 1.0)
        g.build_preconditioner()
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 1.0)
    rng = np.random.default_rng(n)
    for lev, m in enumerate(levels):
        x = rng.normal(size=m.n_u)
        yf = fused.vmult(gmg.OP_A, lev, x, gmg.FP32)
        assert rel_err(yf, o.vmult(1, lev, x)) < TOL32 * 10, lev
        assert rel_err(yf, plain.vmult(gmg.OP_A, lev, x, gmg.FP32)) < TOL32, lev
        assert np.array_equal(yf, fused.vmult(gmg.OP_A, lev, x, gmg.FP32))
    r = rng.normal(size=f.n_u)
    assert rel_err(fused.vcycle(0, r, gmg.FP32), plain.vcycle(0, r, gmg.FP32)) < 1e-5
    rhs = np.concatenate([rng.normal(size=f.n_u), np.zeros(f.n_p)])  # consistent: no pressure load
    rhs[f.constraints_u.rows] = 0.0
    xf, of = fused.solve(rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    xp, op = plain.solve(rhs, linear_solver_tolerance=1e-8, mg_precision=gmg.FP32)
    assert of["status"] == 0 and abs(of["cheap_iterations"] - op["cheap_iterations"]) <= 1
    assert np.linalg.norm(rhs - o.vmult(0, len(levels) - 1, xf)) <= 1.01 * of["solver_tolerance"]


@pytest.mark.parametrize("dim", [2, 3])
def test_caller_geometry_table(dim):
    """GB_GMG_GEOM_TABLE: the caller's inverse Jacobians and |det J| at the
    quadrature points. (a) Built from the level's own Q2 mapping it gives the
    GB_GMG_GEOM_Q2 operators to rounding. (b) From a mapping the Q2 support
    points cannot represent -- the exact Jacobian of a smoothly distorted box,
    x -> x + d(x) on top of the cell's affine map -- the GPU operators agree with
    the oracle given the same table."""
    n = 8 if dim == 2 else 4
    base = mesh.box_hierarchy(dim, n)
    dist = mesh.smooth_distortion(0.05)
    q2 = [mesh.to_q2_geometry(l, dist) for l in base]
    tab = [mesh.to_table_geometry(l) for l in q2]
    eta = random_eta(base[-1], True)
    rng = np.random.default_rng(11)

    def solver(levels):
        g = gmg.StokesMatrixFreeGPU(dim, len(levels))
        g.setup_dofs(levels)
        g.assemble(eta, 0, 1.3, 1)
        return g

    ga, gb = solver(q2), solver(tab)
    for lev, m in enumerate(q2):
        x = rng.normal(size=m.n_u + m.n_p)
        for op in range(4):
            src = x if op == 0 else (x[: m.n_u] if op == 1 else x[m.n_u:])
            assert rel_err(gb.vmult(op, lev, src), ga.vmult(op, lev, src)) < 1e-12, (lev, op)
    # exact Jacobian of X(xi) = B(xi) + d(B(xi)), B the cell's affine box map
    from aspect_gb300 import fe
    gp = fe.tensor_points(dim, fe.gauss(3)[0])
    exact = []
    for m in base:
        xb = m.map_points(gp)
        JB = m.jacobians(gp)
        eps = 1e-6
        grad_d = np.zeros(xb.shape + (dim,))
        for e in range(dim):
            dx = np.zeros(dim)
            dx[e] = eps
            grad_d[..., e] = (dist((xb + dx).reshape(-1, dim)) - dist((xb - dx).reshape(-1, dim))).reshape(
                xb.shape) / (2 * eps)
        exact.append(mesh.to_table_geometry(m, np.einsum("cqij,cqjk->cqik", np.eye(dim) + grad_d, JB)))
    g = solver(exact)
    o = Oracle(exact)
    o.set_viscosity(eta, 0, 1.3, 1)
    for lev, m in enumerate(exact):
        x = rng.normal(size=m.n_u + m.n_p)
        for op in range(4):
            src = x if op == 0 else (x[: m.n_u] if op == 1 else x[m.n_u:])
            assert rel_err(g.vmult(op, lev, src), o.vmult(op, lev, src)) < TOL64, (lev, op)
