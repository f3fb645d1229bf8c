"""Adaptively refined box meshes with hanging nodes (caller side of the boundary).

Stands in for what deal.II's parallel::distributed::Triangulation,
DoFTools::make_hanging_node_constraints and VectorTools::
compute_no_normal_flux_constraints give ASPECT on an adaptive box
(source/simulator/solver/stokes_matrix_free_global_coarsening.cc:1456-1636):
per level, the Q2 velocity / Q1 pressure DoF maps of the active cells, the
hanging-node lines (a hanging node is interpolated from the face or edge nodes
of the coarser neighbour, Q2 for velocity, Q1 for pressure), the no-normal-flux
lines of the box faces, closed so that no master is itself constrained.

Cells are leaves of an octree (quadtree in 2D) over the unit box: (depth,
i, j[, k]) with 0 <= i < 2^depth. Refinement keeps a 2:1 balance across faces
and (in 3D) edges, so hanging nodes only sit on faces and edges of a neighbour
one level coarser.

Level hierarchy: level l is the mesh with every cell deeper than a depth cap
replaced by its ancestor at the cap; caps run from the finest depth down to 0.
Capping keeps the 2:1 balance. A cell of level l either has a parent on level
l-1 (its ancestor one level up; child index = position bits) or is itself a cell
of level l-1 (child index 255).
"""
from __future__ import annotations

import itertools

import numpy as np

from . import fe
from .mesh import GEOM_BOX, Constraints, LevelMesh

SAME_CELL = 255


# ------------------------------------------------------------------ octree
def _cut_by_sphere(cells: np.ndarray, dim: int, center, radius: float) -> np.ndarray:
    """cells: (n, 1+dim) int array (depth, idx...). True where the sphere surface
    passes through the closed cell box."""
    d = cells[:, 0].astype(float)
    h = 1.0 / 2.0 ** d
    lo = cells[:, 1:] * h[:, None]
    hi = lo + h[:, None]
    c = np.asarray(center)[None, :dim]
    nearest = np.clip(c, lo, hi)
    dmin = np.sqrt(np.sum((nearest - c) ** 2, 1))
    far = np.maximum(np.abs(lo - c), np.abs(hi - c))
    dmax = np.sqrt(np.sum(far ** 2, 1))
    return (dmin < radius) & (dmax > radius)


def _children(cell: tuple, dim: int):
    d, idx = cell[0], cell[1:]
    for bits in itertools.product((0, 1), repeat=dim):
        yield (d + 1,) + tuple(2 * i + b for i, b in zip(idx, bits[::-1]))


def _neighbour_offsets(dim: int):
    """Face and (3D) edge neighbour offsets: 1 .. dim-1 non-zero entries."""
    out = []
    for off in itertools.product((-1, 0, 1), repeat=dim):
        nz = sum(1 for o in off if o)
        if 1 <= nz <= max(dim - 1, 1):
            out.append(off)
    return out


def balance(leaves: set, dim: int) -> set:
    """Refine until every face/edge neighbour differs by at most one level."""
    offs = _neighbour_offsets(dim)
    while True:
        to_refine = set()
        for cell in leaves:
            d, idx = cell[0], cell[1:]
            if d < 2:
                continue
            n = 1 << d
            for off in offs:
                nb = tuple(i + o for i, o in zip(idx, off))
                if any(x < 0 or x >= n for x in nb):
                    continue
                for dd in range(d - 2, -1, -1):
                    anc = (dd,) + tuple(x >> (d - dd) for x in nb)
                    if anc in leaves:
                        to_refine.add(anc)
                        break
        if not to_refine:
            return leaves
        for c in to_refine:
            leaves.discard(c)
            leaves.update(_children(c, dim))


def sphere_refined_leaves(dim: int, base_depth: int, n_adaptive: int, center, radius: float) -> set:
    """Uniform mesh of depth base_depth, then n_adaptive rounds of refining the
    cells cut by the sphere |x - center| = radius, each followed by 2:1 balancing."""
    n = 1 << base_depth
    leaves = {(base_depth,) + idx[::-1] for idx in itertools.product(range(n), repeat=dim)}
    for _ in range(n_adaptive):
        arr = np.array(sorted(leaves), dtype=np.int64)
        cut = _cut_by_sphere(arr, dim, center, radius)
        for row in arr[cut]:
            c = tuple(int(v) for v in row)
            leaves.discard(c)
            leaves.update(_children(c, dim))
        leaves = balance(leaves, dim)
    return leaves


def cap_leaves(leaves: set, cap: int) -> list:
    """The mesh with every cell deeper than `cap` replaced by its ancestor at `cap`."""
    out = set()
    for c in leaves:
        d = c[0]
        if d <= cap:
            out.add(c)
        else:
            out.add((cap,) + tuple(x >> (d - cap) for x in c[1:]))
    return sorted(out)


# ------------------------------------------------------------------ DoFs and constraints
def _lagrange_weights(nodes, x):
    return fe.lagrange_1d(np.asarray(nodes, float), np.atleast_1d(x))[0]


class _Lattice:
    """Integer lattice of spacing 1 / 2^(D+1) on which every Q2 node of a mesh
    of maximal depth D lies; points are keyed by a single int64."""

    def __init__(self, dim: int, max_depth: int):
        self.dim = dim
        self.D = max_depth
        self.N = (1 << (max_depth + 1)) + 1

    def key(self, pts: np.ndarray) -> np.ndarray:
        k = np.zeros(pts.shape[:-1], dtype=np.int64)
        for e in reversed(range(self.dim)):
            k = k * self.N + pts[..., e]
        return k

    def size(self, depth: np.ndarray) -> np.ndarray:
        return 1 << (self.D + 1 - depth)


def _cell_node_points(cells: np.ndarray, lat: _Lattice, q: int) -> np.ndarray:
    """Lattice coordinates of the q^dim lexicographic nodes of each cell
    (q = 3: Q2 nodes at 0, S/2, S; q = 2: vertices)."""
    dim = lat.dim
    S = lat.size(cells[:, 0])
    loc = np.array(list(itertools.product(range(q), repeat=dim)))[:, ::-1]  # x fastest
    step = S // (q - 1)
    return cells[:, None, 1:] * S[:, None, None] + loc[None, :, :] * step[:, None, None]


def _hanging_lines(cells: np.ndarray, lat: _Lattice, node_keys: np.ndarray, q: int) -> dict:
    """point key -> [(master key, weight)] for nodes of finer cells that lie on a
    face (or edge) of a coarser cell without being one of its nodes. q = 3 for
    the Q2 velocity nodes, 2 for the Q1 pressure vertices."""
    dim = lat.dim
    sub = 2 * (q - 1)  # candidate resolution on a face: S / sub
    lines = {}
    S_all = lat.size(cells[:, 0])
    for e in range(dim):
        others = [a for a in range(dim) if a != e]
        grid = list(itertools.product(range(sub + 1), repeat=dim - 1))
        cand = [g for g in grid if any(v % 2 for v in g)]  # not a node of the coarse face
        mnodes = list(itertools.product(range(q), repeat=dim - 1))
        w = np.array([[np.prod([_lagrange_weights(np.linspace(0, 1, q), gi / sub)[mi]
                                for gi, mi in zip(g, m)]) for m in mnodes] for g in cand])
        for side in (0, 1):
            ok = S_all >= sub
            cs = cells[ok]
            S = S_all[ok]
            base = cs[:, 1:] * S[:, None]
            base[:, e] += side * S
            for ci, g in enumerate(cand):
                pts = base.copy()
                for a, gi in zip(others, g):
                    pts[:, a] += gi * S // sub
                keys = lat.key(pts)
                pos = np.searchsorted(node_keys, keys)
                pos = np.minimum(pos, len(node_keys) - 1)
                hit = node_keys[pos] == keys
                for r in np.nonzero(hit)[0]:
                    k = int(keys[r])
                    if k in lines:
                        continue
                    ent = []
                    for mi, m in enumerate(mnodes):
                        if abs(w[ci, mi]) < 1e-14:
                            continue
                        mp = base[r].copy()
                        for a, mv in zip(others, m):
                            mp[a] += mv * S[r] // (q - 1)
                        ent.append((int(lat.key(mp[None, :])[0]), float(w[ci, mi])))
                    lines[k] = ent
    return lines


def _close(lines: dict) -> dict:
    """Substitute constrained masters until every master is unconstrained."""
    for _ in range(16):
        changed = False
        for row, (ent, b) in list(lines.items()):
            if not any(m in lines for m, _ in ent):
                continue
            acc, bb = {}, b
            for m, w in ent:
                if m in lines:
                    sub_ent, sub_b = lines[m]
                    bb += w * sub_b
                    for mm, ww in sub_ent:
                        acc[mm] = acc.get(mm, 0.0) + w * ww
                else:
                    acc[m] = acc.get(m, 0.0) + w
            lines[row] = ([(m, w) for m, w in sorted(acc.items()) if abs(w) > 1e-14], bb)
            changed = True
        if not changed:
            return lines
    raise RuntimeError("constraint chains did not close")


def level_mesh(cells: list, dim: int, max_depth: int, free_slip: bool = True) -> LevelMesh:
    """Q2-Q1 DoF maps, box geometry and closed constraints of one adaptive mesh."""
    lat = _Lattice(dim, max_depth)
    arr = np.array(cells, dtype=np.int64)
    n_cells = len(arr)
    vpts = _cell_node_points(arr, lat, 3)
    vkeys = lat.key(vpts)
    node_keys = np.unique(vkeys)
    n_nodes = len(node_keys)
    node_of_cell = np.searchsorted(node_keys, vkeys)  # (n_cells, 3^dim)
    cell_dofs_u = np.concatenate([node_of_cell + c * n_nodes for c in range(dim)], axis=1).astype(np.int32)
    ppts = _cell_node_points(arr, lat, 2)
    pkeys_cell = lat.key(ppts)
    pnode_keys = np.unique(pkeys_cell)
    cell_dofs_p = np.searchsorted(pnode_keys, pkeys_cell).astype(np.int32)

    def coords(keys):
        out = np.zeros((len(keys), dim), dtype=np.int64)
        k = keys.copy()
        for e in range(dim):
            out[:, e] = k % lat.N
            k //= lat.N
        return out

    nxyz = coords(node_keys)
    pxyz = coords(pnode_keys)
    unit = 1.0 / (lat.N - 1)

    # velocity: hanging lines for every component, then no-normal-flux (wins)
    hang = _hanging_lines(arr, lat, node_keys, 3)
    lines = {}
    for k, ent in hang.items():
        node = int(np.searchsorted(node_keys, k))
        m_idx = [(int(np.searchsorted(node_keys, m)), w) for m, w in ent]
        for c in range(dim):
            lines[c * n_nodes + node] = ([(c * n_nodes + m, w) for m, w in m_idx], 0.0)
    if free_slip:
        for c in range(dim):
            on_face = (nxyz[:, c] == 0) | (nxyz[:, c] == lat.N - 1)
            for node in np.nonzero(on_face)[0]:
                lines[int(c * n_nodes + node)] = ([], 0.0)
    lines = _close(lines)
    cu = Constraints.from_dict(lines)
    # pressure: hanging lines only
    phang = _hanging_lines(arr, lat, pnode_keys, 2)
    plines = {}
    for k, ent in phang.items():
        node = int(np.searchsorted(pnode_keys, k))
        plines[node] = ([(int(np.searchsorted(pnode_keys, m)), w) for m, w in ent], 0.0)
    plines = _close(plines)
    cp = Constraints.from_dict(plines)

    h = 1.0 / (1 << arr[:, 0]).astype(float)
    geom = np.concatenate([arr[:, 1:] * h[:, None], np.repeat(h[:, None], dim, 1)], axis=1)
    return LevelMesh(dim=dim, n_cells=n_cells, n_u=dim * n_nodes, n_p=len(pnode_keys),
                     cell_dofs_u=cell_dofs_u, cell_dofs_p=cell_dofs_p, geom_kind=GEOM_BOX, geometry=geom,
                     constraints_u=cu, constraints_p=cp,
                     dof_points_u=np.tile(nxyz * unit, (dim, 1)),
                     dof_component_u=np.repeat(np.arange(dim), n_nodes),
                     dof_points_p=pxyz * unit, cell_level=arr[:, 0].astype(np.int32))


def hierarchy(leaves: set, dim: int, free_slip: bool = True) -> list:
    """Capped-depth global-coarsening hierarchy of an adaptive mesh (see module doc)."""
    max_depth = max(c[0] for c in leaves)
    caps = list(range(0, max_depth + 1))
    cell_lists = [cap_leaves(leaves, c) for c in caps]
    levels = [level_mesh(cl, dim, max_depth, free_slip) for cl in cell_lists]
    for l in range(1, len(levels)):
        coarse_index = {c: i for i, c in enumerate(cell_lists[l - 1])}
        cap = caps[l]
        par = np.zeros(len(cell_lists[l]), np.int32)
        ch = np.zeros(len(cell_lists[l]), np.uint8)
        for i, c in enumerate(cell_lists[l]):
            if c[0] == cap:
                p = (cap - 1,) + tuple(x >> 1 for x in c[1:])
                par[i] = coarse_index[p]
                ch[i] = sum((x & 1) << e for e, x in enumerate(c[1:]))
            else:
                par[i] = coarse_index[c]
                ch[i] = SAME_CELL
        levels[l].parent = par
        levels[l].child_index = ch
    return levels
