"""Finite-element basics for the caller side of the Q2-Q1 Stokes path.

Everything here is textbook mathematics (Lagrange polynomials on the unit
interval, Gauss-Legendre rules), used by the host-side harness that stands in
for deal.II: right-hand-side assembly, error norms, viscosity averaging.

Conventions shared with the C ABI (``include/gb_gmg.h``):

* velocity: FE_Q(2)^dim with 1D nodes {0, 1/2, 1}; cell-local index
  ``c * 3**dim + lex(i, j, k)`` with x fastest;
* pressure: FE_Q(1) with 1D nodes {0, 1}; cell-local index ``lex(i, j, k)``;
* quadrature: QGauss(3) per direction (``QGauss<1>(degree_v+1)`` as in
  source/simulator/solver/stokes_matrix_free_local_smoothing.cc:1657), points
  numbered lexicographically with x fastest.
"""
from __future__ import annotations

import itertools
import numpy as np

Q2_NODES = np.array([0.0, 0.5, 1.0])
Q1_NODES = np.array([0.0, 1.0])
# FE_Q(3): deal.II's default support points are the Gauss-Lobatto points
Q3_NODES = np.array([0.0, 0.5 - 0.5 / np.sqrt(5.0), 0.5 + 0.5 / np.sqrt(5.0), 1.0])


def velocity_nodes(degree: int) -> np.ndarray:
    """1D support points of the velocity element FE_Q(degree) (degree 2 or 3)."""
    return {2: Q2_NODES, 3: Q3_NODES}[degree]


def pressure_nodes(degree: int) -> np.ndarray:
    """1D support points of the pressure element FE_Q(degree - 1)."""
    return {2: Q1_NODES, 3: Q2_NODES}[degree]


def gauss(n: int) -> tuple[np.ndarray, np.ndarray]:
    """n-point Gauss-Legendre rule mapped to [0, 1]."""
    x, w = np.polynomial.legendre.leggauss(n)
    return 0.5 * (x + 1.0), 0.5 * w


def lagrange_1d(nodes: np.ndarray, x: np.ndarray, deriv: int = 0) -> np.ndarray:
    """Values (or first derivatives) of the Lagrange basis on ``nodes`` at ``x``.

    Returns an array of shape (len(x), len(nodes))."""
    x = np.atleast_1d(np.asarray(x, dtype=float))
    n = len(nodes)
    out = np.zeros((len(x), n))
    for i in range(n):
        others = [nodes[m] for m in range(n) if m != i]
        denom = np.prod([nodes[i] - o for o in others])
        if deriv == 0:
            v = np.ones_like(x)
            for o in others:
                v = v * (x - o)
            out[:, i] = v / denom
        else:
            v = np.zeros_like(x)
            for skip in range(len(others)):
                t = np.ones_like(x)
                for m, o in enumerate(others):
                    if m != skip:
                        t = t * (x - o)
                v = v + t
            out[:, i] = v / denom
    return out


def tensor_points(dim: int, pts1d: np.ndarray) -> np.ndarray:
    """Tensor-product points, lexicographic with x fastest: shape (n**dim, dim)."""
    grids = list(itertools.product(range(len(pts1d)), repeat=dim))
    # itertools varies the last index fastest; reverse to make x fastest.
    return np.array([[pts1d[g[dim - 1 - d]] for d in range(dim)] for g in grids])


def tensor_weights(dim: int, w1d: np.ndarray) -> np.ndarray:
    grids = list(itertools.product(range(len(w1d)), repeat=dim))
    return np.array([np.prod([w1d[gi] for gi in g]) for g in grids])


def shape_values(dim: int, nodes: np.ndarray, pts: np.ndarray) -> np.ndarray:
    """Tensor-product Lagrange values at reference points: (n_pts, n_nodes**dim)."""
    n = len(nodes)
    vals = [lagrange_1d(nodes, pts[:, d]) for d in range(dim)]
    out = np.ones((pts.shape[0], n ** dim))
    for idx in range(n ** dim):
        ii = [(idx // n ** d) % n for d in range(dim)]
        for d in range(dim):
            out[:, idx] *= vals[d][:, ii[d]]
    return out


def shape_grads(dim: int, nodes: np.ndarray, pts: np.ndarray) -> np.ndarray:
    """Reference gradients: (n_pts, n_nodes**dim, dim)."""
    n = len(nodes)
    vals = [lagrange_1d(nodes, pts[:, d]) for d in range(dim)]
    ders = [lagrange_1d(nodes, pts[:, d], 1) for d in range(dim)]
    out = np.ones((pts.shape[0], n ** dim, dim))
    for idx in range(n ** dim):
        ii = [(idx // n ** d) % n for d in range(dim)]
        for g in range(dim):
            for d in range(dim):
                out[:, idx, g] *= (ders[d] if d == g else vals[d])[:, ii[d]]
    return out


def quadrature(dim: int, n1d: int) -> tuple[np.ndarray, np.ndarray]:
    p, w = gauss(n1d)
    return tensor_points(dim, p), tensor_weights(dim, w)
