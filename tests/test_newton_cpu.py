"""Newton-derivative terms of the outer Stokes operator in the oracle, checked
against the mathematics they linearise (matrix_free_operators.cc:400-538).

For a viscosity eta(eps, p) = eta0 (1 + eps:eps)^m exp(alpha p) the residual
R(u, p) = K(eta(eps(u), p)) [u; p] has the derivative
    dR [du; dp] = K(eta) [du; dp] + 2 (D : eps(du)) (E : eps(v)) + 2 (deta/dp dp) (E : eps(v))
with E = eps(u), D = deta/deps -- the plain (non-symmetrised) Newton operator
with the strain-rate, Newton-factor and pressure-derivative tables; compressible
adds -2/3 tr(E) (D : eps(du)) I. The reference gives the pressure-derivative
term no such deviatoric correction, so with compressibility its operator is the
exact derivative only for a pressure-independent viscosity (alpha = 0 below).
A central difference of R must match the oracle's Newton operator to O(h^2).
The symmetrised variant (plain and with averaged factors) is checked for
symmetry of its velocity block; the GPU kernels are checked against this
oracle for every variant (test_gpu_newton.py)."""
import numpy as np
import pytest

from aspect_gb300 import mesh
from oracle import Oracle
from tests import numpy_reference as nr


def _sym(t):
    """Full (.., d, d) tensors -> deal.II's unrolled symmetric components."""
    d = t.shape[-1]
    idx = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)] if d == 3 else [(0, 0), (1, 1), (0, 1)]
    return np.stack([t[..., a, b] for a, b in idx], axis=-1)


def _fields(level, x):
    """eps(u) (n_cells, nq, d, d) and p (n_cells, nq) at the Gauss points."""
    d = level.dim
    nv = 3 ** d
    grad, psi, _ = nr.element_data(level, None)
    u = x[: level.n_u][level.cell_dofs_u].reshape(level.n_cells, d, nv)
    p = x[level.n_u:][level.cell_dofs_p]
    G = np.einsum("ckn,cqne->cqke", u, grad)
    return 0.5 * (G + np.swapaxes(G, 2, 3)), np.einsum("cn,qn->cq", p, psi)


ETA0, M_EXP = 1.3, -0.3


def _eta(eps, p, alpha):
    ee = np.einsum("cqab,cqab->cq", eps, eps)
    return ETA0 * (1.0 + ee) ** M_EXP * np.exp(alpha * p), ee


def _residual(levels, x, compressible, alpha):
    o = Oracle(levels)
    eps, p = _fields(levels[-1], x)
    eta, _ = _eta(eps, p, alpha)
    o.set_viscosity(eta, 0, 1.0, compressible)
    return o.vmult(0, len(levels) - 1, x)


@pytest.mark.parametrize("dim,n,compressible", [(2, 4, 0), (2, 4, 1), (3, 2, 0), (3, 2, 1)])
def test_newton_operator_is_the_residual_derivative(dim, n, compressible):
    levels = mesh.box_hierarchy(dim, n)
    f = levels[-1]
    rng = np.random.default_rng(dim * 10 + compressible)
    x = 0.3 * rng.normal(size=f.n_u + f.n_p)
    dx = rng.normal(size=f.n_u + f.n_p)
    for r in f.constraints_u.rows:
        x[r] = dx[r] = 0.0
    alpha = 0.0 if compressible else 0.2
    eps, p = _fields(f, x)
    eta, ee = _eta(eps, p, alpha)
    D = ETA0 * M_EXP * (1.0 + ee)[..., None, None] ** (M_EXP - 1) * 2.0 * eps * np.exp(alpha * p)[..., None, None]
    o = Oracle(levels)
    o.set_viscosity(eta, 0, 1.0, compressible)
    o.set_newton_terms(newton=True, strain_rate=_sym(eps), d_eta_d_strain_rate=_sym(D), d_eta_d_pressure=alpha * eta)
    jd = o.vmult(0, len(levels) - 1, dx)
    h = 1e-5
    fd = (_residual(levels, x + h * dx, compressible, alpha) -
          _residual(levels, x - h * dx, compressible, alpha)) / (2 * h)
    assert np.linalg.norm(jd - fd) <= 1e-7 * np.linalg.norm(fd)


def _tables(f, rng, average=False):
    d = f.dim
    nq = 3 ** d
    ns = 6 if d == 3 else 3
    t = dict(strain_rate=rng.normal(size=(f.n_cells, nq, ns)), d_eta_d_strain_rate=rng.normal(size=(f.n_cells, nq, ns)),
             d_eta_d_pressure=rng.normal(size=(f.n_cells, nq)), dilation_lhs=rng.normal(size=(f.n_cells, nq)),
             d_dilation_d_strain_rate=rng.normal(size=(f.n_cells, nq, ns)),
             d_dilation_d_pressure=rng.normal(size=(f.n_cells, nq)))
    if average:  # the same values at every point of a cell
        for k, v in t.items():
            t[k] = np.repeat(v[:, :1], nq, axis=1)
    return t


@pytest.mark.parametrize("dim,compressible,average", [(2, 0, False), (3, 1, False), (3, 0, True), (2, 1, True)])
def test_symmetrized_newton_velocity_block_is_symmetric(dim, compressible, average):
    levels = mesh.box_hierarchy(dim, 2)
    f = levels[-1]
    rng = np.random.default_rng(5)
    t = _tables(f, rng)
    t["d_eta_d_strain_rate"] = t["strain_rate"] * 0.7  # a symmetric Newton form needs D parallel to E
    o = Oracle(levels)
    o.set_viscosity(np.exp(rng.uniform(-1, 1, size=(f.n_cells, 3 ** dim))), 0, 1.0, compressible)
    o.set_newton_terms(newton=True, symmetrize=True, average=average, **{k: t[k] for k in
                       ("strain_rate", "d_eta_d_strain_rate", "d_eta_d_pressure")})
    a, b = rng.normal(size=f.n_u), rng.normal(size=f.n_u)
    a[f.constraints_u.rows] = 0.0
    b[f.constraints_u.rows] = 0.0
    z = np.zeros(f.n_p)
    ya = o.vmult(0, len(levels) - 1, np.concatenate([a, z]))[: f.n_u]
    yb = o.vmult(0, len(levels) - 1, np.concatenate([b, z]))[: f.n_u]
    assert abs(b @ ya - a @ yb) <= 1e-12 * abs(b @ ya)

