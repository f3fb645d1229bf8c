"""Free-surface stabilisation term of the outer Stokes operator in the oracle
(StokesOperator::local_apply_boundary_face, matrix_free_operators.cc:563-602):
    dst_u(phi) += int_F -(T . u) (n . phi) dS
on the listed boundary faces, checked (1) against the dense face matrix of the
numpy reference assembled with the constraints, on lattice, distorted Q2 and
hanging-node levels, and (2) against closed-form surface integrals: with
T = (0, .., t) on the top face of the unit box, x^T K_fs x = -t int_top u_z^2.
The harness's face normals times JxW are checked on the unit box and on the
outer sphere of a shell (area 4 pi R^2, normal x/|x|)."""
import numpy as np
import pytest

from aspect_gb300 import mesh, octree
from oracle import Oracle
from tests import numpy_reference as nr


def _levels(case):
    if case == "box3d":
        return mesh.box_hierarchy(3, 4, open_faces=(5,))
    if case == "box2d":
        return mesh.box_hierarchy(2, 8, open_faces=(3,))
    if case == "q2-distorted2d":
        return [mesh.to_q2_geometry(l, mesh.smooth_distortion()) for l in mesh.box_hierarchy(2, 8, open_faces=(3,))]
    leaves = octree.sphere_refined_leaves(2, 3, 1, (0.5, 0.9), 0.2)
    return octree.hierarchy(leaves, 2, free_slip=False)  # hanging nodes on the open top


def _top(level):
    d = level.dim - 1
    return mesh.boundary_faces(level, lambda x: np.abs(x[:, d] - 1.0) < 1e-9)


@pytest.mark.parametrize("case", ["box3d", "box2d", "q2-distorted2d", "adaptive2d"])
def test_oracle_face_term_matches_dense(case):
    levels = _levels(case)
    f = levels[-1]
    fc, fn = _top(f)
    assert len(fc) > 0
    rng = np.random.default_rng(3)
    T = rng.normal(size=(len(fc), 3 ** (f.dim - 1), f.dim))
    nj = mesh.face_normal_jxw(f, fc, fn)
    o = Oracle(levels)
    o.set_viscosity(np.exp(rng.uniform(-1, 1, size=(f.n_cells,))), 0, 1.0)
    x = rng.normal(size=f.n_u + f.n_p)
    top = len(levels) - 1
    y0 = o.vmult(0, top, x)
    o.set_free_surface(fc, fn, T)
    y1 = o.vmult(0, top, x)
    K = nr.free_surface_matrix(f, fc, fn, T, nj)
    C = nr.constraint_matrix(f.n_u, f.constraints_u)
    ref = C.T @ (K @ (C @ x[: f.n_u]))
    mask = f.constraints_u.constrained_mask(f.n_u)
    ref[mask] = 0.0
    dy = y1 - y0
    assert np.linalg.norm(dy[: f.n_u] - ref) <= 1e-13 * np.linalg.norm(ref)
    assert np.all(dy[f.n_u:] == 0.0)
    o.set_free_surface()
    assert np.array_equal(o.vmult(0, top, x), y0)


@pytest.mark.parametrize("dim", [2, 3])
def test_face_term_closed_form(dim):
    """u_z = 1 + x y (3D) / u_y = 1 + x^2 (2D), exact in Q2, on the open top face of
    the unit box: x^T K_fs x = -t int_top u_z^2 dS = -t (1 + 1/2 + 1/9) / -t 28/15."""
    levels = mesh.box_hierarchy(dim, 4, open_faces=(2 * dim - 1,))
    f = levels[-1]
    fc, fn = _top(f)
    t = 0.37
    T = np.zeros((len(fc), 3 ** (dim - 1), dim))
    T[..., dim - 1] = t
    o = Oracle(levels)
    o.set_viscosity(np.ones(f.n_cells), 0, 1.0)
    o.set_free_surface(fc, fn, T)
    x = np.zeros(f.n_u + f.n_p)
    pts, comp = f.dof_points_u, f.dof_component_u
    vert = comp == dim - 1
    val = 1 + pts[:, 0] * pts[:, 1] if dim == 3 else 1 + pts[:, 0] ** 2
    x[: f.n_u][vert] = val[vert]
    x[: f.n_u][f.constraints_u.constrained_mask(f.n_u)] = 0.0
    top = len(levels) - 1
    o2 = Oracle(levels)
    o2.set_viscosity(np.ones(f.n_cells), 0, 1.0)
    q = x[: f.n_u] @ (o.vmult(0, top, x) - o2.vmult(0, top, x))[: f.n_u]
    exact = -t * ((1 + 0.5 + 1.0 / 9.0) if dim == 3 else 28.0 / 15.0)
    assert abs(q - exact) <= 1e-12 * abs(exact)


def test_face_normals_on_box_and_sphere():
    f = mesh.box_hierarchy(3, 4)[-1]
    for fno in range(6):
        d, side = divmod(fno, 2)
        fc, fn = mesh.boundary_faces(f, lambda x, d=d, side=side: np.abs(x[:, d] - side) < 1e-12)
        nj = mesh.face_normal_jxw(f, fc, fn)
        expect = np.zeros(3)
        expect[d] = 1.0 if side else -1.0
        assert np.allclose(nj.sum(axis=(0, 1)), expect, atol=1e-14)
    from aspect_gb300 import shell
    s = shell.hierarchy(1, 3, 0.55, 1.0)[-1]
    fc, fn = mesh.boundary_faces(s, lambda x: np.abs(np.linalg.norm(x, axis=1) - 1.0) < 1e-9)
    nj = mesh.face_normal_jxw(s, fc, fn)
    area = np.linalg.norm(nj, axis=-1).sum()
    assert abs(area - 4 * np.pi) < 2e-3 * 4 * np.pi
    xq = np.concatenate([s.map_points(mesh.face_reference_points(3, int(k))[0])[c][None]
                         for c, k in zip(fc, fn)])
    cosang = np.einsum("fqi,fqi->fq", nj, xq) / (np.linalg.norm(nj, axis=-1) * np.linalg.norm(xq, axis=-1))
    assert cosang.min() > 0.999
