"""Brute-force assembled operators in numpy (test helper).

Element matrices are formed from the textbook bilinear forms at QGauss(3),
assembled into dense global matrices and reduced with the constraints
(K_c = C^T K C on unconstrained DoFs, identity on constrained rows) -- the
matrix that deal.II's MatrixFreeOperators::Base::vmult applies. Small meshes only.
"""
import numpy as np

from aspect_gb300 import fe


def constraint_matrix(n, cons):
    """C: (n x n) with x_full = C x_unconstrained-part (constrained columns unused)."""
    C = np.eye(n)
    for i, r in enumerate(cons.rows):
        C[r, :] = 0.0
        a, b = cons.ptr[i], cons.ptr[i + 1]
        for c, w in zip(cons.cols[a:b], cons.weights[a:b]):
            C[r, c] += w
    return C


def element_data(level, eta_cell_q):
    dim, deg = level.dim, getattr(level, "degree", 2)
    pts, w = fe.quadrature(dim, deg + 1)
    G = fe.shape_grads(dim, fe.velocity_nodes(deg), pts)  # (nq, nv, dim) reference
    psi = fe.shape_values(dim, fe.pressure_nodes(deg), pts)
    J = level.jacobians(pts)  # (nc, nq, dim, dim)
    invJ = np.linalg.inv(J)
    jxw = np.abs(np.linalg.det(J)) * w[None, :]
    grad = np.einsum("qna,cqae->cqne", G, invJ)  # real gradients
    return grad, psi, jxw


def stokes_blocks(level, eta_q, s, compressible=False):
    """Dense A (n_u x n_u), B^T-part (n_u x n_p: -s p div v), M (n_p x n_p: s^2/eta)."""
    dim = level.dim
    nv = (getattr(level, "degree", 2) + 1) ** dim
    grad, psi, jxw = element_data(level, eta_q)
    A = np.zeros((level.n_u, level.n_u))
    BT = np.zeros((level.n_u, level.n_p))
    M = np.zeros((level.n_p, level.n_p))
    for c in range(level.n_cells):
        # symmetric gradient of each velocity basis function: (nq, dim*nv, dim, dim)
        E = np.zeros((grad.shape[1], dim * nv, dim, dim))
        for comp in range(dim):
            for n in range(nv):
                g = grad[c, :, n, :]  # (nq, dim)
                T = np.zeros((grad.shape[1], dim, dim))
                T[:, comp, :] = g
                E[:, comp * nv + n] = 0.5 * (T + T.transpose(0, 2, 1))
        div = np.trace(E, axis1=2, axis2=3)
        eta = eta_q[c]
        Ke = np.einsum("q,qiab,qjab->ij", 2 * eta * jxw[c], E, E)
        if compressible:
            Ke -= np.einsum("q,qi,qj->ij", 2 * eta * jxw[c] / 3, div, div)
        Be = np.einsum("q,qi,qn->in", -s * jxw[c], div, psi)
        Me = np.einsum("q,qm,qn->mn", s * s / eta * jxw[c], psi, psi)
        du, dp = level.cell_dofs_u[c], level.cell_dofs_p[c]
        A[np.ix_(du, du)] += Ke
        BT[np.ix_(du, dp)] += Be
        M[np.ix_(dp, dp)] += Me
    return A, BT, M


def constrained_operator(K, C_row, C_col, mask_row=None, identity=True):
    R = C_row.T @ K @ C_col
    if identity and mask_row is not None:
        R[mask_row, :] = 0.0
        R[:, mask_row] = 0.0
        R[mask_row, mask_row] = 1.0
    return R


def free_surface_matrix(level, face_cell, face_no, stab, normal_jxw):
    """Dense velocity matrix (caller numbering, no constraints) of the free-surface
    face term: K[i, j] = sum_faces sum_q -(T_q . phi_j(x_q)) (nJxW_q . phi_i(x_q))."""
    from aspect_gb300 import mesh
    dim = level.dim
    nv = 3 ** dim
    K = np.zeros((level.n_u, level.n_u))
    for f, (c, fno) in enumerate(zip(face_cell, face_no)):
        pts, _ = mesh.face_reference_points(dim, int(fno))
        phi = fe.shape_values(dim, fe.Q2_NODES, pts)  # (nq, nv)
        dofs = level.cell_dofs_u[c].reshape(dim, nv)
        for q in range(len(pts)):
            for a in range(dim):
                for b in range(dim):
                    coef = -stab[f, q, b] * normal_jxw[f, q, a]
                    K[np.ix_(dofs[a], dofs[b])] += coef * np.outer(phi[q], phi[q])
    return K
