"""Synthetic Stokes problems and the caller-side steps around one solve.

These functions stand in for the parts of ASPECT that sit *around* the
matrix-free solver and stay on the caller's side of the C ABI:

* right-hand side ``rho g . phi_u`` (source/simulator/assemblers/stokes.cc:285-400),
  condensed with the constraints as ``distribute_local_to_global`` does;
* pressure scaling = volume-weighted geometric mean viscosity at cell
  midpoints / length scale (source/simulator/helper_functions.cc:255-345;
  box length scale 0.01 * x-extent, source/geometry_model/box.cc:252-255);
* viscosity averaging (include/aspect/material_model/interface.h:818-831);
* surface pressure normalisation (source/simulator/helper_functions.cc:765-880);
* error norms of the SolCx postprocessor (benchmarks/solcx/solcx.h:3106-3190,
  QGauss(degree_v+2)).

Random inputs use one SplitMix64 stream per seed; the default seed of the
benchmark workloads is 20261204 + workload index.
"""
from __future__ import annotations

import dataclasses
import math
import numpy as np

from . import fe
from .mesh import LevelMesh, box_hierarchy

BASE_SEED = 20261204


class SplitMix64:
    def __init__(self, seed: int):
        self.state = seed & 0xFFFFFFFFFFFFFFFF

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
        return z ^ (z >> 31)

    def uniform(self, n: int = 1) -> np.ndarray:
        return np.array([(self.next_u64() >> 11) * (1.0 / 9007199254740992.0) for _ in range(n)])

    def normal(self, n: int) -> np.ndarray:
        u1 = np.maximum(self.uniform(n), 1e-300)
        u2 = self.uniform(n)
        return np.sqrt(-2 * np.log(u1)) * np.cos(2 * np.pi * u2)


@dataclasses.dataclass
class StokesProblem:
    """Everything one solve needs, in the caller's (deal.II-like) numbering."""

    name: str
    levels: list
    eta: np.ndarray            # finest level: [n_cells] (averaged) or [n_cells, n_q]
    projection: int            # 0: DGQ0 level tables, 1: DGQ1 (project to Q1)
    pressure_scaling: float
    rhs: np.ndarray            # [n_u + n_p], condensed
    gravity_dir: int           # for reporting only
    extra: dict = dataclasses.field(default_factory=dict)

    @property
    def fine(self) -> LevelMesh:
        return self.levels[-1]

    @property
    def n_dofs(self) -> int:
        return self.fine.n_u + self.fine.n_p


def q_points_real(level: LevelMesh, n1d: int = 3) -> tuple[np.ndarray, np.ndarray]:
    """Real quadrature points (n_cells, n_q, dim) and JxW (n_cells, n_q)."""
    pts, w = fe.quadrature(level.dim, n1d)
    x = level.map_points(pts)
    J = level.jacobians(pts)
    det = np.linalg.det(J)
    return x, np.abs(det) * w[None, :]


def assemble_rhs(level: LevelMesh, force_q: np.ndarray) -> np.ndarray:
    """f_u = int force . phi_u over QGauss(degree+1); force_q: (n_cells, n_q, dim).
    Pressure block zero (incompressible). Condensed with the constraints."""
    dim, deg = level.dim, level.degree
    pts, w = fe.quadrature(dim, deg + 1)
    phi = fe.shape_values(dim, fe.velocity_nodes(deg), pts)  # (nq, nv)
    _, jxw = q_points_real(level, deg + 1)
    nv = (deg + 1) ** dim
    f = np.zeros(level.n_u + level.n_p)
    loc = np.einsum("cqd,qn,cq->cdn", force_q, phi, jxw).reshape(level.n_cells, dim * nv)
    np.add.at(f, level.cell_dofs_u.ravel(), loc.ravel())
    fu = f[: level.n_u]
    level.constraints_u.condense(fu)
    f[: level.n_u] = fu
    return f


def pressure_scaling(level: LevelMesh, eta_mid: np.ndarray, length_scale: float) -> float:
    """Geometric mean of the midpoint viscosity (volume weighted) / length scale."""
    pts = np.full((1, level.dim), 0.5)
    J = level.jacobians(pts)
    vol = np.abs(np.linalg.det(J))[:, 0]
    return float(np.exp(np.sum(np.log(eta_mid) * vol) / np.sum(vol)) / length_scale)


def harmonic_average(eta_q: np.ndarray) -> np.ndarray:
    """Cellwise harmonic average over the quadrature points, unweighted as
    MaterialAveraging computes it (source/material_model/interface.cc:576-595:
    N / sum 1/eta_q, zero if any value is zero)."""
    with np.errstate(divide="ignore"):
        avg = eta_q.shape[1] / np.sum(1.0 / eta_q, 1)
    return np.where(np.any(eta_q == 0.0, 1), 0.0, avg)


def normalize_pressure_surface(level: LevelMesh, p: np.ndarray, top: float = 1.0) -> float:
    """Shift p so that its mean over the top boundary (x_{dim-1} == top) is zero.
    Returns the adjustment added. Exact for Q1 on straight faces."""
    dim = level.dim
    g = level.geometry.reshape(level.n_cells, -1)
    num = den = 0.0
    if level.geom_kind != 0:
        raise NotImplementedError("surface normalisation implemented for box cells only")
    on_top = np.abs(g[:, dim - 1] + g[:, 2 * dim - 1] - top) < 1e-12
    # top face local pressure nodes: those with bit (dim-1) set
    loc = [n for n in range(2 ** dim) if (n >> (dim - 1)) & 1]
    for c in np.nonzero(on_top)[0]:
        area = np.prod(g[c, dim:2 * dim - 1])
        num += area * np.mean(p[level.cell_dofs_p[c, loc]])
        den += area
    adj = -num / den
    p += adj
    return adj


def normalize_pressure_volume(level: LevelMesh, p: np.ndarray) -> float:
    pts, w = fe.quadrature(level.dim, 3)
    psi = fe.shape_values(level.dim, fe.Q1_NODES, pts)
    _, jxw = q_points_real(level)
    pq = np.einsum("qn,cn->cq", psi, p[level.cell_dofs_p])
    adj = -np.sum(pq * jxw) / np.sum(jxw)
    p += adj
    return adj


def evaluate_fields(level: LevelMesh, u: np.ndarray, p: np.ndarray, n1d: int):
    """Velocity and pressure at QGauss(n1d) points: (n_cells, nq, dim), (n_cells, nq)."""
    dim, deg = level.dim, level.degree
    pts, w = fe.quadrature(dim, n1d)
    phi = fe.shape_values(dim, fe.velocity_nodes(deg), pts)
    psi = fe.shape_values(dim, fe.pressure_nodes(deg), pts)
    nv = (deg + 1) ** dim
    ul = u[level.cell_dofs_u].reshape(level.n_cells, dim, nv)
    uq = np.einsum("qn,cdn->cqd", phi, ul)
    pq = np.einsum("qn,cn->cq", psi, p[level.cell_dofs_p])
    return uq, pq


def error_norms(level: LevelMesh, u, p, exact_u_q, exact_p_q, n1d: int = 4):
    """(u_L1, p_L1, u_L2, p_L2) against exact values at the QGauss(n1d) points.
    The L1 norm of a vector field sums the absolute values of its components,
    as VectorTools::integrate_difference does for L1_norm."""
    uq, pq = evaluate_fields(level, u, p, n1d)
    pts, w = fe.quadrature(level.dim, n1d)
    J = level.jacobians(pts)
    jxw = np.abs(np.linalg.det(J)) * w[None, :]
    du = uq - exact_u_q
    dp = pq - exact_p_q
    u_l1 = np.sum(np.sum(np.abs(du), -1) * jxw)
    p_l1 = np.sum(np.abs(dp) * jxw)
    u_l2 = math.sqrt(np.sum(np.sum(du ** 2, -1) * jxw))
    p_l2 = math.sqrt(np.sum(dp ** 2 * jxw))
    return u_l1, p_l1, u_l2, p_l2


# --------------------------------------------------------------------- problems
def solcx(n_refinements: int, eta_B: float = 1e6, density_sign: float = -1.0,
          name: str | None = None, average_density: bool = False) -> StokesProblem:
    """SolCx (benchmarks/solcx/solcx.h:2953-2975): eta = 1 for x < 1/2 and eta_B
    otherwise, rho = density_sign * sin(pi y) cos(pi x), g = (0, -1), free slip on
    all walls, harmonic averaging (constant per cell here). density_sign = -1 is
    the reference benchmark; +1 is the variant of the 64x64 workload.
    average_density: the density is harmonically averaged per cell too (the
    reference's "harmonic average" as opposed to "harmonic average only
    viscosity")."""
    n = 2 ** n_refinements
    levels = box_hierarchy(2, n)
    fine = levels[-1]
    xq, jxw = q_points_real(fine)
    eta_q = np.where(xq[..., 0] < 0.5, 1.0, eta_B)
    eta = harmonic_average(eta_q)
    rho = density_sign * np.sin(np.pi * xq[..., 1]) * np.cos(np.pi * xq[..., 0])
    if average_density:
        rho = np.repeat(harmonic_average(rho)[:, None], rho.shape[1], 1)
    force = np.zeros(xq.shape)
    force[..., 1] = -rho
    rhs = assemble_rhs(fine, force)
    mid = fine.map_points(np.full((1, 2), 0.5))[:, 0, :]
    s = pressure_scaling(fine, np.where(mid[:, 0] < 0.5, 1.0, eta_B), 0.01 * 1.0)
    return StokesProblem(name or f"solcx_{n}x{n}", levels, eta, 0, s, rhs, 1)


def nsinker(n_refinements: int, centres: np.ndarray, dynamic_viscosity_ratio: float = 1e4,
            sinker_density: float = 10.0, delta: float = 200.0, omega: float = 0.1,
            averaging: str = "harmonic") -> StokesProblem:
    """The reference's NSinker benchmark material on the unit cube
    (benchmarks/nsinker/nsinker.cc:61-76 evaluate, :280-313 inside_outside_factor;
    parameters of benchmarks/nsinker/nsinker_gmg.prm): with chi the product over
    the sinkers of 1 - exp(-delta max(0, |x - c| - omega/2)^2),
    eta = (sqrt(r) - 1/sqrt(r)) (1 - chi) + 1/sqrt(r) for the viscosity ratio r and
    rho = sinker_density (1 - chi), per quadrature point; eta harmonically averaged
    per cell ("harmonic average only viscosity"), rho not averaged; gravity -z of
    magnitude 1; zero velocity on all six faces; pressure scaling 1 (the benchmark
    overrides it, nsinker.cc:320-331). The sinker centres are data of the
    benchmark, passed in by the caller. averaging = "none": the viscosity stays
    per quadrature point on the finest level and the level tables are the
    cellwise (DGQ0) projection, as the reference does without averaging
    (matrix_free_operators.cc:137-330, stokes_matrix_free_local_smoothing.cc:104-116)."""
    n = 2 ** n_refinements
    levels = box_hierarchy(3, n, no_slip=True)
    fine = levels[-1]
    xq, jxw = q_points_real(fine)
    chi = np.ones(xq.shape[:-1])
    for c in np.asarray(centres, float):
        dist = np.linalg.norm(xq - c, axis=-1)
        chi *= 1.0 - np.exp(-delta * np.maximum(0.0, dist - omega / 2.0) ** 2)
    sr = math.sqrt(dynamic_viscosity_ratio)
    eta_q = (sr - 1.0 / sr) * (1.0 - chi) + 1.0 / sr
    rho = sinker_density * (1.0 - chi)
    force = np.zeros(xq.shape)
    force[..., 2] = -rho
    rhs = assemble_rhs(fine, force)
    eta = eta_q if averaging == "none" else harmonic_average(eta_q)
    return StokesProblem(f"nsinker_{n}^3", levels, eta, 0, 1.0, rhs, 2, extra=dict(eta_q=eta_q))


def sinker_centres(seed: int, n: int = 8) -> np.ndarray:
    rng = SplitMix64(seed)
    return 0.2 + 0.6 * rng.uniform(3 * n).reshape(n, 3)


def sinker_viscosity(x: np.ndarray, centres: np.ndarray, eta_min: float = 1e-6) -> np.ndarray:
    """eta = eta_min + (1 - eta_min) prod_i (1 - exp(-d_i^2 / (2 0.05^2))): the
    smooth-sinker formula with its contrast parameter set to 1e6 (eta_min = 1e-6,
    range 1e-6 .. 1)."""
    prod = np.ones(x.shape[:-1])
    for c in centres:
        d2 = np.sum((x - c) ** 2, -1)
        prod *= 1.0 - np.exp(-d2 / (2 * 0.05 ** 2))
    return eta_min + (1 - eta_min) * prod


def sinker_density(x: np.ndarray, centres: np.ndarray, radius: float = 0.075) -> np.ndarray:
    inside = np.zeros(x.shape[:-1], bool)
    for c in centres:
        inside |= np.sum((x - c) ** 2, -1) < radius ** 2
    return inside.astype(float)


def sinkers_3d(n: int = 32, seed: int = BASE_SEED + 2, projection: int = 1,
               n_coarse: int = 1, degree: int = 2) -> StokesProblem:
    """3D unit cube, n^3 Q2-Q1 cells, 8 smooth sinkers (centres seeded uniform in
    [0.2, 0.8]^3), eta = 1e-6 + (1-1e-6) prod_i(...) (1e6 contrast), rho = 1
    inside r = 0.075, g = -z,
    free slip. ``projection`` = 1 uses ASPECT's default averaging for GMG
    (project to Q1 only viscosity: per-quadrature-point viscosity); 0 uses the
    harmonic cell average. ``degree`` 3: Q3-Q2 elements, QGauss(4)."""
    levels = box_hierarchy(3, n, n_coarse=n_coarse, degree=degree)
    fine = levels[-1]
    centres = sinker_centres(seed)
    xq, jxw = q_points_real(fine, degree + 1)
    eta_q = sinker_viscosity(xq, centres)
    eta = eta_q if projection == 1 else harmonic_average(eta_q)
    rho = sinker_density(xq, centres)
    force = np.zeros(xq.shape)
    force[..., 2] = -rho
    rhs = assemble_rhs(fine, force)
    mid = fine.map_points(np.full((1, 3), 0.5))[:, 0, :]
    s = pressure_scaling(fine, sinker_viscosity(mid, centres), 0.01)
    name = f"sinkers_{n}^3" + ("" if degree == 2 else f"_Q{degree}Q{degree - 1}")
    return StokesProblem(name, levels, eta, projection, s, rhs, 2, extra=dict(centres=centres, seed=seed))


def adaptive_sphere(base_depth: int = 4, n_adaptive: int = 2, radius: float = 0.2,
                    eta_in: float = 1e3, drho: float = 0.01) -> StokesProblem:
    """3D unit cube, uniform depth base_depth (16^3 for 4) plus n_adaptive rounds
    of refining the cells cut by the sphere |x - (1/2,1/2,1/2)| = radius, with 2:1
    face/edge balance (hanging nodes). eta = eta_in and rho = 1 + drho inside the
    sphere, eta = rho = 1 outside, evaluated per quadrature point with the Q1
    projection; g = -z; free slip."""
    from . import octree
    leaves = octree.sphere_refined_leaves(3, base_depth, n_adaptive, (0.5, 0.5, 0.5), radius)
    levels = octree.hierarchy(leaves, 3)
    fine = levels[-1]
    xq, jxw = q_points_real(fine)
    inside = np.sum((xq - 0.5) ** 2, -1) < radius ** 2
    eta = np.where(inside, eta_in, 1.0)
    rho = np.where(inside, 1.0 + drho, 1.0)
    force = np.zeros(xq.shape)
    force[..., 2] = -rho
    rhs = assemble_rhs(fine, force)
    mid = fine.map_points(np.full((1, 3), 0.5))[:, 0, :]
    s = pressure_scaling(fine, np.where(np.sum((mid - 0.5) ** 2, -1) < radius ** 2, eta_in, 1.0), 0.01)
    return StokesProblem(f"adaptive_sphere_{2 ** base_depth}^3+{n_adaptive}", levels, eta, 1, s, rhs, 2,
                         extra=dict(cells_per_depth={int(d): int(np.sum(fine.cell_level == d))
                                                     for d in np.unique(fine.cell_level)}))


def real_spherical_harmonics_field(x: np.ndarray, max_degree: int, seed: int) -> np.ndarray:
    """sum_{l=1..max_degree} sum_m c_lm Y_lm(theta, phi) with seeded standard-normal
    coefficients, real harmonics P_l^|m|(cos theta) {cos, sin}(|m| phi) normalised
    per (l, m); returned divided by its maximum modulus over the points."""
    from scipy.special import lpmv
    r = np.linalg.norm(x, axis=-1)
    ct = np.clip(x[..., 2] / r, -1, 1)
    phi = np.arctan2(x[..., 1], x[..., 0])
    rng = SplitMix64(seed)
    out = np.zeros(x.shape[:-1])
    for l in range(1, max_degree + 1):
        for m in range(-l, l + 1):
            c = rng.normal(1)[0]
            am = abs(m)
            norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.factorial(l - am) / math.factorial(l + am))
            ang = np.cos(am * phi) if m >= 0 else np.sin(am * phi)
            out += c * norm * lpmv(am, l, ct) * ang
    return out / np.abs(out).max()


def spherical_shell(n_refinements: int = 3, Ra: float = 1e5, contrast: float = 1e4,
                    amplitude: float = 0.01, max_degree: int = 8, seed: int = BASE_SEED + 3,
                    r_in: float = 0.55, r_out: float = 1.0, n_adaptive: int = 0,
                    refinement_fraction: float = 0.3) -> StokesProblem:
    """Spherical shell r in [0.55, 1], the 96-cell cube-sphere refined n times,
    T = conductive profile + amplitude sin(pi (r-r_in)/(r_out-r_in)) Y(theta, phi)
    with Y a seeded real spherical-harmonic field of degree <= 8, eta =
    exp(-ln(contrast) T) per quadrature point (Q1 projection), buoyancy
    Ra T r_hat, free slip on both spheres (rotation null space).

    n_adaptive rounds of refinement on the temperature gradient follow the global
    ones: cell indicator |grad T(centre)| sqrt(|K|) (an L2 norm of grad T over the
    cell at one point), the cells holding `refinement_fraction` of the indicator
    sum refined (ASPECT's default fixed-fraction strategy with fraction 0.3);
    hanging nodes on the coarse/fine interfaces."""
    from . import shell

    def temperature(x, r):
        t = (1 / r - 1 / r_out) / (1 / r_in - 1 / r_out)
        env = np.sin(np.pi * (r - r_in) / (r_out - r_in))
        return t + amplitude * env * real_spherical_harmonics_field(x, max_degree, seed)

    if n_adaptive == 0:
        levels = shell.hierarchy(n_refinements, 4, r_in, r_out)
    else:
        cells = shell.all_cells(4, n_refinements)
        for _ in range(n_adaptive):
            arr = np.array(cells, dtype=np.int64)
            xc = shell.cell_centres(cells, 4, r_in, r_out)
            rc = np.linalg.norm(xc, axis=-1)
            hgt = 1e-6
            st = np.concatenate([xc[None]] + [xc[None] + s * hgt * np.eye(3)[e] for e in range(3) for s in (1, -1)])
            Ts = temperature(st.reshape(-1, 3), np.linalg.norm(st.reshape(-1, 3), axis=-1)).reshape(7, -1)
            grad = np.stack([(Ts[1 + 2 * e] - Ts[2 + 2 * e]) / (2 * hgt) for e in range(3)], -1)
            d = arr[:, 1]
            vol = rc ** 2 * (1.0 / (4 * (1 << d))) ** 2 * ((r_out - r_in) / (1 << d))
            cells = shell.refine_fixed_fraction(cells, np.linalg.norm(grad, axis=-1) * np.sqrt(vol),
                                                refinement_fraction)
        levels = shell.adaptive_hierarchy(cells, 4, r_in, r_out)
    fine = levels[-1]
    xq, jxw = q_points_real(fine)
    r = np.linalg.norm(xq, axis=-1)

    T = temperature(xq, r)
    eta = np.exp(-math.log(contrast) * T)
    force = Ra * T[..., None] * xq / r[..., None]
    rhs = assemble_rhs(fine, force)
    mid = fine.map_points(np.full((1, 3), 0.5))[:, 0, :]
    rm = np.linalg.norm(mid, axis=-1)
    length = 1e4 / (6336000.0 - 3481000.0) * (r_out - r_in)
    s = pressure_scaling(fine, np.exp(-math.log(contrast) * temperature(mid, rm)), length)
    name = f"spherical_shell_ref{n_refinements}" + (f"+{n_adaptive}" if n_adaptive else "")
    return StokesProblem(name, levels, eta, 1, s, rhs, -1, extra=dict(temperature_q=T))
