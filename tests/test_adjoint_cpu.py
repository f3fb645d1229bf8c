"""Adjoint gradient maths on the CPU oracle (no GPU): the gradient formula
-int_c 2 eta eps(u):eps(lambda) against central finite differences of the misfit."""
import numpy as np

from aspect_gb300 import adjoint
from oracle import Oracle


class OracleEvaluator:
    def __init__(self, base, top, u_obs):
        self.base, self.top, self.u_obs = base, top, u_obs
        self.o = Oracle(base.levels)

    def solve(self, lneta, rhs):
        self.o.set_viscosity(np.exp(lneta), 0, self.base.pressure_scaling)
        self.o.build_preconditioner(False)
        x, info = self.o.solve(rhs, tol_rel=1e-13)
        assert info["status"] == 0
        return x

    def J(self, lneta):
        x = self.solve(lneta, self.base.rhs)
        return adjoint.misfit(x[: self.base.fine.n_u], self.u_obs, self.top), x

    def gradient(self, lneta):
        J, x = self.J(lneta)
        n_u = self.base.fine.n_u
        lam = self.solve(lneta, adjoint.misfit_gradient_u(x[:n_u], self.u_obs, self.top, len(self.base.rhs)))
        return J, self.o.adjoint_gradient(x[:n_u], lam[:n_u])


def test_random_field_statistics():
    f = adjoint.gaussian_random_field(16, 0.1, 1.0, adjoint.SEED_A)
    assert abs(f.mean()) < 1e-12 and abs(f.std() - 1.0) < 1e-12
    g = adjoint.gaussian_random_field(16, 0.1, 1.0, adjoint.SEED_B)
    assert abs(np.corrcoef(f, g)[0, 1]) < 0.2


def test_oracle_adjoint_gradient_matches_finite_differences():
    n = 4
    base = adjoint.base_problem(n)
    top = adjoint.top_face_dofs(base.fine)
    ev = OracleEvaluator(base, top, np.zeros(base.fine.n_u))
    _, x_obs = ev.J(adjoint.gaussian_random_field(n, 0.1, 1.0, adjoint.SEED_B))
    ev.u_obs = x_obs[: base.fine.n_u].copy()
    lneta = adjoint.gaussian_random_field(n, 0.1, 1.0, adjoint.SEED_A)
    J, g = ev.gradient(lneta)
    assert J > 0
    eps = 1e-6
    dirs = adjoint.fd_directions(base.fine.n_cells, 4, 7)
    fd = np.array([(ev.J(lneta + eps * d)[0] - ev.J(lneta - eps * d)[0]) / (2 * eps) for d in dirs])
    gd = dirs @ g
    assert np.linalg.norm(fd - gd) <= 1e-5 * np.linalg.norm(gd), (fd, gd)
