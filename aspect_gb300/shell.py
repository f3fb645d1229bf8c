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
from .octree import SAME_CELL, _close

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

    # velocity: hanging lines for every component, then no-normal-flux (wins for
    # the component it constrains, as the no-normal-flux lines are entered first
    # at source/simulator/solver/stokes_matrix_free_global_coarsening.cc:1570-1589)
    mixed = arr[:, 1].min() != arr[:, 1].max()
    lines = {}
    if mixed:
        for node, ent in _hanging(arr, m, r_in, r_out, uniq, node_of_cell, 3).items():
            for c in range(3):
                lines[c * n_nodes + node] = ([(c * n_nodes + mm, w) for mm, w in ent], 0.0)
    if free_slip:
        r = np.linalg.norm(node_x, axis=1)
        on_bnd = (np.abs(r - r_in) < 1e-9) | (np.abs(r - r_out) < 1e-9)
        for node in np.nonzero(on_bnd)[0]:
            n = node_x[node] / r[node]
            c = int(np.argmax(np.abs(n)))
            ent = [(int(e * n_nodes + node), float(-n[e] / n[c])) for e in range(3)
                   if e != c and abs(n[e]) > 1e-14]
            lines[int(c * n_nodes + node)] = (ent, 0.0)
    if mixed:
        lines = _close(lines)
    cu = Constraints.from_dict(lines)
    cp = Constraints.empty()
    if mixed:
        ph = _hanging(arr, m, r_in, r_out, puniq, cell_dofs_p, 2)
        cp = Constraints.from_dict(_close({node: (ent, 0.0) for node, ent in ph.items()}))
    return LevelMesh(dim=3, n_cells=n_cells, n_u=3 * n_nodes, n_p=len(puniq), cell_dofs_u=cell_dofs_u,
                     cell_dofs_p=cell_dofs_p, geom_kind=GEOM_Q2, geometry=X.reshape(n_cells, 81),
                     constraints_u=cu, constraints_p=cp,
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


# ------------------------------------------------------------------ adaptive shells
def refine_fixed_fraction(cells: list, indicator: np.ndarray, fraction: float) -> list:
    """One round of refinement: the cells with the largest indicators that together
    hold `fraction` of the indicator sum are replaced by their 8 children (the
    refinement half of deal.II's refine_and_coarsen_fixed_fraction, as called at
    source/simulator/core.cc:1785 with "Refinement fraction" = 0.3 by default,
    source/simulator/parameters.cc:917). Refining one round from a uniform mesh
    keeps the 2:1 balance."""
    order = np.argsort(-indicator, kind="stable")
    cum = np.cumsum(indicator[order])
    n = int(np.searchsorted(cum, fraction * cum[-1])) + 1
    flag = np.zeros(len(cells), bool)
    flag[order[:n]] = True
    out = []
    for c, f in zip(cells, flag):
        if not f:
            out.append(c)
            continue
        p, d, i, j, k = c
        for b in range(8):
            out.append((p, d + 1, 2 * i + (b & 1), 2 * j + ((b >> 1) & 1), 2 * k + ((b >> 2) & 1)))
    return out


def cell_centres(cells: list, m: int = 4, r_in: float = R_INNER, r_out: float = R_OUTER) -> np.ndarray:
    arr = np.array(cells, dtype=np.int64)
    d = arr[:, 1]
    ha, hr = 1.0 / (m * (1 << d)), 1.0 / (1 << d)
    return shell_points(arr[:, 0], (arr[:, 2] + 0.5) * ha, (arr[:, 3] + 0.5) * ha, (arr[:, 4] + 0.5) * hr,
                        r_in, r_out)


def _surface_candidates(q: int):
    """Reference points on the surface of the unit cell at which a neighbour one
    level finer has nodes that this cell has not (q = 3: Q2 nodes, spacing 1/4;
    q = 2: Q1 vertices, spacing 1/2), with their Lagrange weights over the cell's
    q^3 lexicographic nodes."""
    sub = 2 * (q - 1)
    pts, wts = [], []
    nodes = np.linspace(0.0, 1.0, q)
    for g in itertools.product(range(sub + 1), repeat=3):
        g = g[::-1]  # x fastest
        if not any(v in (0, sub) for v in g) or not any(v % 2 for v in g):
            continue
        xi = np.array(g, float) / sub
        l = [fe_lagrange(nodes, x) for x in xi]
        w = np.einsum("k,j,i->kji", l[2], l[1], l[0]).ravel()
        pts.append(xi)
        wts.append(w)
    return np.array(pts), np.array(wts)


def fe_lagrange(nodes: np.ndarray, x: float) -> np.ndarray:
    out = np.ones(len(nodes))
    for a in range(len(nodes)):
        for b in range(len(nodes)):
            if a != b:
                out[a] *= (x - nodes[b]) / (nodes[a] - nodes[b])
    return out


def _row_ids(*arrays):
    """Common integer ids of the int64 rows of several (n_i, 3) arrays."""
    allr = np.concatenate(arrays, axis=0)
    _, inv = np.unique(allr, axis=0, return_inverse=True)
    inv = inv.ravel()
    out, s = [], 0
    for a in arrays:
        out.append(inv[s:s + len(a)])
        s += len(a)
    return out


def _hanging(arr: np.ndarray, m: int, r_in: float, r_out: float, node_keys: np.ndarray,
             node_of_cell: np.ndarray, q: int) -> dict:
    """node -> [(master node, weight)]: nodes of finer cells on a face or edge of a
    coarser cell that are not nodes of it, interpolated from that cell's nodes in
    its reference coordinates (what DoFTools::make_hanging_node_constraints gives:
    Q2 face/edge interpolation for velocity, Q1 for pressure). Points are matched
    by their physical keys, so patch boundaries need no special case."""
    coarse = np.nonzero(arr[:, 1] < arr[:, 1].max())[0]
    if len(coarse) == 0:
        return {}
    xi, w = _surface_candidates(q)
    cs = arr[coarse]
    d = cs[:, 1]
    ha, hr = 1.0 / (m * (1 << d)), 1.0 / (1 << d)
    u = (cs[:, None, 2] + xi[None, :, 0]) * ha[:, None]
    v = (cs[:, None, 3] + xi[None, :, 1]) * ha[:, None]
    ww = (cs[:, None, 4] + xi[None, :, 2]) * hr[:, None]
    patch = np.repeat(cs[:, 0], len(xi))
    X = shell_points(patch, u.ravel(), v.ravel(), ww.ravel(), r_in, r_out)
    ckeys = _keys(X)
    nid, cid = _row_ids(node_keys, ckeys)
    lookup = -np.ones(max(int(nid.max()), int(cid.max())) + 1, np.int64)
    lookup[nid] = np.arange(len(node_keys))
    hit_node = lookup[cid].reshape(len(coarse), len(xi))
    lines = {}
    for r, t in zip(*np.nonzero(hit_node >= 0)):
        node = int(hit_node[r, t])
        if node in lines:
            continue
        masters = node_of_cell[coarse[r]]
        lines[node] = [(int(masters[n]), float(w[t, n])) for n in range(len(masters)) if abs(w[t, n]) > 1e-14]
    return lines


def adaptive_hierarchy(leaves: list, m: int = 4, r_in: float = R_INNER, r_out: float = R_OUTER,
                       free_slip: bool = True) -> list:
    """Capped-depth global-coarsening hierarchy of an adaptive shell: level l is the
    mesh with every cell deeper than l replaced by its ancestor at depth l. A cell
    of level l has a parent on level l-1 (child index = position bits) or is a
    cell of level l-1 itself (child index SAME_CELL)."""
    max_depth = max(c[1] for c in leaves)

    def cap(c, depth):
        p, d, i, j, k = c
        s = max(d - depth, 0)
        return (p, min(d, depth), i >> s, j >> s, k >> s)

    cell_lists = [sorted({cap(c, l) for c in leaves}) for l in range(max_depth + 1)]
    levels = [level_mesh(cl, m, r_in, r_out, free_slip) for cl in cell_lists]
    for l in range(1, len(levels)):
        index = {c: i for i, c in enumerate(cell_lists[l - 1])}
        par = np.zeros(len(cell_lists[l]), np.int32)
        ch = np.zeros(len(cell_lists[l]), np.uint8)
        for n, c in enumerate(cell_lists[l]):
            p, d, i, j, k = c
            if d == l:
                par[n] = index[(p, d - 1, i >> 1, j >> 1, k >> 1)]
                ch[n] = (i & 1) | ((j & 1) << 1) | ((k & 1) << 2)
            else:
                par[n] = index[c]
                ch[n] = SAME_CELL
        levels[l].parent = par
        levels[l].child_index = ch
    return levels
