"""Spherical-shell meshes (caller side of the boundary).

Stands in for ASPECT's spherical shell geometry with deal.II's 96-cell
``GridGenerator::hyper_shell`` (source/geometry_model/spherical_shell.cc:361-373)
refined globally, a Q2 mapping whose support points lie on the spheres, and
``VectorTools::compute_no_normal_flux_constraints`` on both surfaces.

Cells: an equiangular cube-sphere, 6 patches of m x m angular cells and one
radial layer (m = 4 gives the 96 coarse cells), refined by bisection in all
three parameter directions. A cell (patch, depth, i, j, k) covers
u in [i, i+1] / (m 2^depth), v likewise, w in [k, k+1] / 2^depth of its patch;
its reference directions are (u, v, w), so children of a refined cell follow
the usual child-index bits. Nodes shared by patches are identified by their
physical coordinates.

No-normal-flux: at a boundary node with unit normal n, the component c with the
largest |n_c| is constrained, u_c = -sum_{e != c} (n_e / n_c) u_e (the form
deal.II produces), so the lines couple the components of one node.
"""
from __future__ import annotations

import itertools

import numpy as np

from .mesh import GEOM_Q2, Constraints, LevelMesh

R_INNER = 0.55
R_OUTER = 1.0


def _tan_param(t: np.ndarray) -> np.ndarray:
    a = np.tan((t - 0.5) * (np.pi / 2))
    # tan(+-pi/4) is 1 -/+ 1 ulp: snap so that patch edges coincide exactly
    a = np.where(np.abs(np.abs(a) - 1.0) < 1e-13, np.sign(a), a)
    return np.where(np.abs(a) < 1e-15, 0.0, a)


def directions(patch: np.ndarray, u: np.ndarray, v: np.ndarray) -> np.ndarray:
    """Unit directions of cube-sphere parameter points (vectorised)."""
    a, b = _tan_param(u), _tan_param(v)
    one = np.ones_like(a)
    cand = np.stack([
        np.stack([one, a, b], -1),      # +x
        np.stack([-one, b, a], -1),     # -x
        np.stack([b, one, a], -1),      # +y
        np.stack([a, -one, b], -1),     # -y
        np.stack([a, b, one], -1),      # +z
        np.stack([b, a, -one], -1),     # -z
    ])
    d = cand[patch, np.arange(len(patch))]
    return d / np.linalg.norm(d, axis=1, keepdims=True)


def shell_points(patch, u, v, w, r_in=R_INNER, r_out=R_OUTER) -> np.ndarray:
    r = r_in + w * (r_out - r_in)
    return directions(patch, u, v) * r[:, None]


def all_cells(m: int, depth: int) -> list:
    n_ang = m << depth
    n_rad = 1 << depth
    return [(p, depth, i, j, k) for p in range(6) for k in range(n_rad) for j in range(n_ang)
            for i in range(n_ang)]


def _cell_params(cells: np.ndarray, m: int, q: int):
    """Parameter coordinates (u, v, w) of the q^3 lexicographic nodes of each cell."""
    d = cells[:, 1]
    ha = 1.0 / (m * (1 << d))
    hr = 1.0 / (1 << d)
    loc = np.array(list(itertools.product(range(q), repeat=3)))[:, ::-1] / (q - 1)  # x fastest
    u = (cells[:, None, 2] + loc[None, :, 0]) * ha[:, None]
    v = (cells[:, None, 3] + loc[None, :, 1]) * ha[:, None]
    w = (cells[:, None, 4] + loc[None, :, 2]) * hr[:, None]
    return u, v, w


def _keys(x: np.ndarray) -> np.ndarray:
    """Integer keys of physical points (shared points of different patches agree)."""
    return np.round(x * (1 << 30)).astype(np.int64)


def level_mesh(cells: list, m: int = 4, r_in: float = R_INNER, r_out: float = R_OUTER,
               free_slip: bool = True) -> LevelMesh:
    arr = np.array(cells, dtype=np.int64)
    n_cells = len(arr)
    u, v, w = _cell_params(arr, m, 3)
    patch = np.repeat(arr[:, 0], 27)
    X = shell_points(patch, u.ravel(), v.ravel(), w.ravel(), r_in, r_out)  # (n_cells*27, 3)
    keys = _keys(X)
    uniq, inv = np.unique(keys, axis=0, return_inverse=True)
    inv = inv.ravel()
    n_nodes = len(uniq)
    node_x = np.zeros((n_nodes, 3))
    node_x[inv] = X
    node_of_cell = inv.reshape(n_cells, 27)
    cell_dofs_u = np.concatenate([node_of_cell + c * n_nodes for c in range(3)], axis=1).astype(np.int32)
    corner = [n for n in range(27) if all(((n // 3 ** e) % 3) != 1 for e in range(3))]  # lexicographic corners
    ckeys = keys.reshape(n_cells, 27, 3)[:, corner, :].reshape(-1, 3)
    puniq, pinv = np.unique(ckeys, axis=0, return_inverse=True)
    cell_dofs_p = pinv.ravel().reshape(n_cells, 8).astype(np.int32)
    p_x = np.zeros((len(puniq), 3))
    p_x[pinv.ravel()] = X.reshape(n_cells, 27, 3)[:, corner, :].reshape(-1, 3)

    lines = {}
    if free_slip:
        r = np.linalg.norm(node_x, axis=1)
        on_bnd = (np.abs(r - r_in) < 1e-9) | (np.abs(r - r_out) < 1e-9)
        for node in np.nonzero(on_bnd)[0]:
            n = node_x[node] / r[node]
            c = int(np.argmax(np.abs(n)))
            ent = [(int(e * n_nodes + node), float(-n[e] / n[c])) for e in range(3)
                   if e != c and abs(n[e]) > 1e-14]
            lines[int(c * n_nodes + node)] = (ent, 0.0)
    cu = Constraints.from_dict(lines)
    return LevelMesh(dim=3, n_cells=n_cells, n_u=3 * n_nodes, n_p=len(puniq), cell_dofs_u=cell_dofs_u,
                     cell_dofs_p=cell_dofs_p, geom_kind=GEOM_Q2, geometry=X.reshape(n_cells, 81),
                     constraints_u=cu, constraints_p=Constraints.empty(),
                     dof_points_u=np.tile(node_x, (3, 1)), dof_component_u=np.repeat(np.arange(3), n_nodes),
                     dof_points_p=p_x, cell_level=arr[:, 1].astype(np.int32))


def hierarchy(n_refinements: int, m: int = 4, r_in: float = R_INNER, r_out: float = R_OUTER,
              free_slip: bool = True) -> list:
    """Levels 0 .. n_refinements of the globally refined shell."""
    cell_lists = [all_cells(m, d) for d in range(n_refinements + 1)]
    levels = [level_mesh(cl, m, r_in, r_out, free_slip) for cl in cell_lists]
    for l in range(1, len(levels)):
        index = {c: i for i, c in enumerate(cell_lists[l - 1])}
        par = np.zeros(len(cell_lists[l]), np.int32)
        ch = np.zeros(len(cell_lists[l]), np.uint8)
        for n, (p, d, i, j, k) in enumerate(cell_lists[l]):
            par[n] = index[(p, d - 1, i >> 1, j >> 1, k >> 1)]
            ch[n] = (i & 1) | ((j & 1) << 1) | ((k & 1) << 2)
        levels[l].parent = par
        levels[l].child_index = ch
    return levels


def rotation_modes(level: LevelMesh) -> np.ndarray:
    """The three rigid rotations omega x x at the velocity DoFs (caller numbering),
    the null space that free slip on both spheres leaves in the velocity."""
    n = level.n_u // 3
    x = level.dof_points_u[:n]
    modes = np.zeros((3, level.n_u))
    for a in range(3):
        om = np.zeros(3)
        om[a] = 1.0
        r = np.cross(om, x)
        for c in range(3):
            modes[a, c * n:(c + 1) * n] = r[:, c]
    return modes
