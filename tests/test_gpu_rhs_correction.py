"""correct_stokes_rhs on the GPU (gb_gmg_correct_stokes_rhs) against the dense
assembled form of the reference's correction
(source/simulator/solver/stokes_matrix_free_local_smoothing.cc:618-754):
rhs - C^T K u0, with K the unconstrained Stokes matrix applied to plain values
u0 that are nonzero only at constrained DoFs, C^T distributing contributions of
constrained DoFs to their masters (and dropping Dirichlet ones), so constrained
rows are unchanged. Lattice, indexed and adaptive (hanging-node) levels, per-point
viscosity, incompressible and compressible. Tolerance 1e-12 relative."""
import numpy as np
import pytest

from aspect_gb300 import gmg, octree
from tests import numpy_reference as nr
from tests.gpu_util import hierarchy, random_eta, rel_err

pytestmark = pytest.mark.gpu


def _levels(case):
    if case == "adaptive2d":
        leaves = octree.sphere_refined_leaves(2, 3, 1, (0.5, 0.5), 0.2)
        return octree.hierarchy(leaves, 2)
    dim, n = (3, 4) if case.startswith("box3d") else (2, 8)
    return hierarchy(dim, n)


@pytest.mark.parametrize("case,force,comp", [("box3d", 0, 0), ("box3d", 1, 1), ("box2d", 0, 0),
                                             ("adaptive2d", 0, 1)])
def test_correct_stokes_rhs_matches_assembled(case, force, comp):
    levels = _levels(case)
    f = levels[-1]
    eta = random_eta(f, True)
    s = 1.7
    g = gmg.StokesMatrixFreeGPU(f.dim, len(levels), {"force_indexed_layout": force})
    g.setup_dofs(levels)
    g.assemble(eta, 0, s, comp)
    rng = np.random.default_rng(11)
    mu = f.constraints_u.constrained_mask(f.n_u)
    mp = f.constraints_p.constrained_mask(f.n_p)
    assert mu.any()
    u0 = np.zeros(f.n_u + f.n_p)
    u0[: f.n_u][mu] = rng.normal(size=mu.sum())
    u0[f.n_u:][mp] = rng.normal(size=mp.sum())
    rhs = rng.normal(size=f.n_u + f.n_p)
    got = g.correct_stokes_rhs(u0, rhs)
    A, BT, M = nr.stokes_blocks(f, eta, s, compressible=bool(comp))
    K = np.block([[A, BT], [BT.T, np.zeros((f.n_p, f.n_p))]])
    C = np.zeros((f.n_u + f.n_p, f.n_u + f.n_p))
    C[: f.n_u, : f.n_u] = nr.constraint_matrix(f.n_u, f.constraints_u)
    C[f.n_u:, f.n_u:] = nr.constraint_matrix(f.n_p, f.constraints_p)
    corr = C.T @ (K @ u0)
    ref = rhs - corr
    assert rel_err(got - rhs, -corr) < 1e-12
    assert np.array_equal(got[: f.n_u][mu], rhs[: f.n_u][mu])
    assert rel_err(got, ref) < 1e-12


@pytest.mark.parametrize("case", ["box3d", "box2d", "adaptive2d", "shell"])
def test_body_force_rhs_on_device(case):
    """gb_gmg_assemble_rhs (the rho g . phi_u term of source/simulator/assemblers/
    stokes.cc:285-400, condensed with the constraints) against the harness's numpy
    assembly: lattice, indexed hanging-node and curved Q2 levels, 1e-12."""
    from aspect_gb300 import problems, shell
    if case == "shell":
        levels = shell.hierarchy(1, 4, 0.55, 1.0)
    else:
        levels = _levels(case)
    f = levels[-1]
    rng = np.random.default_rng(4)
    force = rng.normal(size=(f.n_cells, 3 ** f.dim, f.dim))
    g = gmg.StokesMatrixFreeGPU(f.dim, len(levels))
    g.setup_dofs(levels)
    ref = problems.assemble_rhs(f, force)
    got = g.assemble_rhs(force)
    assert rel_err(got, ref) < 1e-12
    assert np.all(got[f.n_u:] == 0.0) and np.all(got[f.constraints_u.rows] == 0.0)
