"""Adjoint viscosity gradient of a surface-velocity misfit (no reference counterpart).

Workload: 3D unit cube, n^3 Q2-Q1 cells, cellwise ln(eta) = seeded Gaussian
random field (correlation length 0.1, standard deviation 1), density of the
8-sinker workload (rho = 1 inside r = 0.075), g = -z, free slip. The observed
velocity u_obs is the forward solution for a second seeded field, and

    J(eta) = 1/2 sum_{i in top-face velocity DoFs} (u_i(eta) - u_obs,i)^2.

The Stokes operator K is symmetric, so the adjoint solve K lambda = dJ/du reuses
the forward GMG solver unchanged. The gradient
dJ/d ln(eta_c) = -int_c 2 eta eps(u) : eps(lambda) comes from the backward kernel
behind gb_gmg_adjoint_gradient.

:class:`StokesMisfit` is a thin torch.autograd.Function over the C ABI (a test
shim: forward = solve + misfit, backward = adjoint solve + backward kernel).
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import problems
from .mesh import box_hierarchy

SEED_A = problems.BASE_SEED + 4
SEED_B = problems.BASE_SEED + 5


def gaussian_random_field(n: int, corr_length: float, std: float, seed: int) -> np.ndarray:
    """Periodic Gaussian random field on the n^3 cell grid of the unit cube,
    Gaussian covariance exp(-r^2 / (2 corr_length^2)), generated by filtering
    SplitMix64 white noise in Fourier space; normalised to zero mean and the
    given standard deviation. Lexicographic cell order (x fastest)."""
    rng = problems.SplitMix64(seed)
    w = rng.normal(n ** 3).reshape(n, n, n)  # [z][y][x]
    k = 2 * np.pi * np.fft.fftfreq(n, d=1.0 / n)
    kz, ky, kx = np.meshgrid(k, k, k, indexing="ij")
    filt = np.exp(-(kx ** 2 + ky ** 2 + kz ** 2) * corr_length ** 2 / 4)
    f = np.real(np.fft.ifftn(np.fft.fftn(w) * filt))
    f = (f - f.mean()) / f.std() * std
    return f.ravel()


@dataclasses.dataclass
class AdjointProblem:
    base: problems.StokesProblem  # mesh, rhs, pressure scaling (eta replaced per evaluation)
    lneta: np.ndarray             # [n_cells] reference field (seed A)
    u_obs: np.ndarray             # [n_u] observed velocity (forward solve with seed B)
    top: np.ndarray               # velocity DoF indices on the top face (unconstrained)


def top_face_dofs(level) -> np.ndarray:
    z = level.dof_points_u[:, level.dim - 1]
    cons = level.constraints_u.constrained_mask(level.n_u)
    return np.nonzero((np.abs(z - 1.0) < 1e-12) & ~cons)[0]


def base_problem(n: int) -> problems.StokesProblem:
    P = problems.sinkers_3d(n, projection=0)
    # pressure scaling of a unit-viscosity reference; fixed for all evaluations
    return dataclasses.replace(P, pressure_scaling=1.0 / 0.01, projection=0)


def misfit(u: np.ndarray, u_obs: np.ndarray, top: np.ndarray) -> float:
    r = u[top] - u_obs[top]
    return 0.5 * float(r @ r)


def misfit_gradient_u(u: np.ndarray, u_obs: np.ndarray, top: np.ndarray, n_total: int) -> np.ndarray:
    g = np.zeros(n_total)
    g[top] = u[top] - u_obs[top]
    return g


class Evaluator:
    """J(ln eta) and dJ/d ln eta through a GPU solver (gmg.StokesMatrixFreeGPU)."""

    def __init__(self, solver, base: problems.StokesProblem, u_obs: np.ndarray, top: np.ndarray,
                 tol: float = 1e-12, mg_precision: int = 1):
        self.g = solver
        self.base = base
        self.u_obs = u_obs
        self.top = top
        self.tol = tol
        self.prec = mg_precision
        self.n_u = base.fine.n_u

    def _set(self, lneta: np.ndarray):
        self.g.assemble(np.exp(lneta), 0, self.base.pressure_scaling)
        self.g.build_preconditioner()

    def forward(self, lneta: np.ndarray, keep_preconditioner: bool = False):
        """J at ln(eta). keep_preconditioner: reuse the preconditioner of the last
        full evaluation (so that the nearby solves of a finite-difference pair
        share it and their iteration errors cancel)."""
        if keep_preconditioner:
            self.g.update_viscosity(np.exp(lneta))
        else:
            self._set(lneta)
        x, out = self.g.solve(self.base.rhs, linear_solver_tolerance=self.tol, mg_precision=self.prec)
        return x, misfit(x[: self.n_u], self.u_obs, self.top), out

    def gradient(self, lneta: np.ndarray):
        """Returns (J, dJ/d ln eta, forward solution, adjoint solution)."""
        x, J, _ = self.forward(lneta)
        rhs_adj = misfit_gradient_u(x[: self.n_u], self.u_obs, self.top, len(self.base.rhs))
        lam, _ = self.g.solve(rhs_adj, linear_solver_tolerance=self.tol, mg_precision=self.prec)
        grad = self.g.adjoint_gradient(x[: self.n_u], lam[: self.n_u])
        return J, grad, x, lam


def make_problem(n: int, solver_factory, tol: float = 1e-12, mg_precision: int = 1):
    """Builds the workload: returns (AdjointProblem, Evaluator)."""
    base = base_problem(n)
    lneta_a = gaussian_random_field(n, 0.1, 1.0, SEED_A)
    lneta_b = gaussian_random_field(n, 0.1, 1.0, SEED_B)
    solver = solver_factory(base)
    top = top_face_dofs(base.fine)
    ev = Evaluator(solver, base, np.zeros(base.fine.n_u), top, tol, mg_precision)
    x_obs, _, _ = ev.forward(lneta_b)
    ev.u_obs = x_obs[: base.fine.n_u].copy()
    return AdjointProblem(base, lneta_a, ev.u_obs, top), ev


def fd_directions(n_cells: int, k: int, seed: int) -> np.ndarray:
    """k seeded random directions, each of unit 2-norm."""
    rng = problems.SplitMix64(seed)
    d = rng.normal(k * n_cells).reshape(k, n_cells)
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def torch_misfit_function():
    """torch.autograd.Function shim: J = StokesMisfit.apply(lneta, evaluator)."""
    import torch

    class StokesMisfit(torch.autograd.Function):
        @staticmethod
        def forward(ctx, lneta, evaluator):
            J, grad, _, _ = evaluator.gradient(lneta.detach().cpu().double().numpy())
            ctx.save_for_backward(torch.as_tensor(grad, dtype=lneta.dtype, device=lneta.device))
            return torch.as_tensor(J, dtype=lneta.dtype, device=lneta.device)

        @staticmethod
        def backward(ctx, gJ):
            (grad,) = ctx.saved_tensors
            return gJ * grad, None

    return StokesMisfit
