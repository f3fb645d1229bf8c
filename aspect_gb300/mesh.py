"""Level meshes, DoF maps and constraints handed to the solver through the C ABI.

This module is the caller side of the boundary: it produces exactly the arrays
that ASPECT's ``setup_dofs`` produces through deal.II
(source/simulator/solver/stokes_matrix_free_global_coarsening.cc:1456-1732 builds
one DoFHandler plus AffineConstraints per level of a global-coarsening
hierarchy): per level, the cell-to-DoF maps of the Q2 velocity and Q1 pressure,
the cell geometry, the constraint lines (no-normal-flux, Dirichlet, hanging
nodes) and the parent/child relation to the next coarser level.

Conventions (shared with ``include/gb_gmg.h``):

* cells of a level are numbered 0..n_cells-1; local DoFs are lexicographic,
  velocity components blocked (``c * 3**dim + node``);
* geometry kind 0 (``GEOM_BOX``): per cell ``[x0.., h..]`` (lower corner and
  edge lengths of an axis-aligned box); kind 1 (``GEOM_Q2``): the 3**dim Q2
  support points of the cell mapping, ``[node][dim]``; kind 2 (``GEOM_TABLE``):
  per QGauss(3) point the inverse Jacobian and ``|det J|`` of the caller's own
  mapping (``to_table_geometry``; the solver only, not the harness's assembly);
* a constraint line is ``x[row] = sum_k w_k x[col_k] + inhomogeneity``; a line
  with no entries is a Dirichlet constraint (zero in the homogeneous operators);
* child index of a fine cell = sum_d bit_d << d, bit_d = which half of the
  parent's reference cell the child occupies in direction d.
"""
from __future__ import annotations

import dataclasses
import itertools
import numpy as np

GEOM_BOX = 0
GEOM_Q2 = 1
GEOM_TABLE = 2


@dataclasses.dataclass
class Constraints:
    """Closed AffineConstraints of one block, in CSR form."""

    rows: np.ndarray  # int32 [n_lines]
    ptr: np.ndarray  # int32 [n_lines+1]
    cols: np.ndarray  # int32 [nnz]
    weights: np.ndarray  # float64 [nnz]
    inhom: np.ndarray  # float64 [n_lines]

    @staticmethod
    def empty() -> "Constraints":
        return Constraints(np.zeros(0, np.int32), np.zeros(1, np.int32), np.zeros(0, np.int32),
                           np.zeros(0), np.zeros(0))

    @staticmethod
    def from_dict(lines: dict) -> "Constraints":
        """``lines``: row -> (list[(col, weight)], inhomogeneity)."""
        rows = np.array(sorted(lines), dtype=np.int32)
        ptr = [0]
        cols, ws, inh = [], [], []
        for r in rows:
            ent, b = lines[int(r)]
            for c, w in ent:
                cols.append(c)
                ws.append(w)
            ptr.append(len(cols))
            inh.append(b)
        return Constraints(rows, np.array(ptr, np.int32), np.array(cols, np.int32),
                           np.array(ws, float), np.array(inh, float))

    @property
    def n_lines(self) -> int:
        return len(self.rows)

    def constrained_mask(self, n: int) -> np.ndarray:
        m = np.zeros(n, bool)
        m[self.rows] = True
        return m

    def distribute(self, x: np.ndarray) -> None:
        """x[row] = sum w x[col] + b (AffineConstraints::distribute)."""
        for i, r in enumerate(self.rows):
            a, b = self.ptr[i], self.ptr[i + 1]
            x[r] = np.dot(self.weights[a:b], x[self.cols[a:b]]) + self.inhom[i]

    def set_zero(self, x: np.ndarray) -> None:
        x[self.rows] = 0.0

    def condense(self, f: np.ndarray) -> None:
        """Move rhs entries of constrained rows to their masters, then zero them."""
        for i, r in enumerate(self.rows):
            a, b = self.ptr[i], self.ptr[i + 1]
            if b > a:
                np.add.at(f, self.cols[a:b], self.weights[a:b] * f[r])
        f[self.rows] = 0.0


@dataclasses.dataclass
class LevelMesh:
    dim: int
    n_cells: int
    n_u: int
    n_p: int
    cell_dofs_u: np.ndarray  # int32 [n_cells, dim*3**dim]
    cell_dofs_p: np.ndarray  # int32 [n_cells, 2**dim]
    geom_kind: int
    geometry: np.ndarray  # float64, see module doc
    constraints_u: Constraints
    constraints_p: Constraints
    parent: np.ndarray | None = None  # int32 [n_cells] into the next coarser level
    child_index: np.ndarray | None = None  # uint8 [n_cells]
    # Position of each velocity / pressure DoF (for boundary conditions and
    # function interpolation); velocity DoF positions repeat per component.
    dof_points_u: np.ndarray | None = None
    dof_component_u: np.ndarray | None = None
    dof_points_p: np.ndarray | None = None
    # Optional extra information used by the harness only.
    cell_level: np.ndarray | None = None
    degree: int = 2  # velocity degree: FE_Q(degree)^dim x FE_Q(degree - 1)

    def q2_support_points(self) -> np.ndarray:
        """Q2 mapping support points per cell, shape (n_cells, 3**dim, dim)."""
        from . import fe
        if self.geom_kind == GEOM_Q2:
            return self.geometry.reshape(self.n_cells, 3 ** self.dim, self.dim)
        ref = fe.tensor_points(self.dim, fe.Q2_NODES)
        g = self.geometry.reshape(self.n_cells, 2 * self.dim)
        return g[:, None, :self.dim] + ref[None, :, :] * g[:, None, self.dim:]

    def map_points(self, ref_pts: np.ndarray) -> np.ndarray:
        """Real coordinates of reference points in every cell: (n_cells, n_pts, dim)."""
        from . import fe
        if self.geom_kind == GEOM_BOX:
            g = self.geometry.reshape(self.n_cells, 2 * self.dim)
            return g[:, None, :self.dim] + ref_pts[None, :, :] * g[:, None, self.dim:]
        phi = fe.shape_values(self.dim, fe.Q2_NODES, ref_pts)
        X = self.q2_support_points()
        return np.einsum("qn,cnd->cqd", phi, X)

    def jacobians(self, ref_pts: np.ndarray) -> np.ndarray:
        """dx/dxi at reference points: (n_cells, n_pts, dim, dim) [x-comp, xi-dir]."""
        from . import fe
        if self.geom_kind == GEOM_BOX:
            g = self.geometry.reshape(self.n_cells, 2 * self.dim)
            J = np.zeros((self.n_cells, len(ref_pts), self.dim, self.dim))
            for d in range(self.dim):
                J[:, :, d, d] = g[:, None, self.dim + d]
            return J
        dphi = fe.shape_grads(self.dim, fe.Q2_NODES, ref_pts)
        X = self.q2_support_points()
        return np.einsum("qne,cnd->cqde", dphi, X)


def face_reference_points(dim: int, face_no: int) -> tuple[np.ndarray, np.ndarray]:
    """QGauss(3) points of a cell face in reference coordinates, (3**(dim-1), dim),
    and their weights: face_no = 2*d + side (xi_d = side); the two tangential axes
    in increasing order, the lower fastest (the C ABI's free-surface point order)."""
    from . import fe
    d, side = divmod(face_no, 2)
    tang = [a for a in range(dim) if a != d]
    g, w = fe.gauss(3)
    pts = np.zeros((3 ** (dim - 1), dim))
    wts = np.ones(3 ** (dim - 1))
    for q in range(3 ** (dim - 1)):
        for m, a in enumerate(tang):
            i = (q // 3 ** m) % 3
            pts[q, a] = g[i]
            wts[q] *= w[i]
        pts[q, d] = side
    return pts, wts


def face_normal_jxw(level: "LevelMesh", face_cell: np.ndarray, face_no: np.ndarray) -> np.ndarray:
    """Outward unit normal times surface JxW at the face points (n_faces, 3**(dim-1), dim),
    from the level's box or Q2 geometry (cross product of the tangential Jacobian columns)."""
    dim = level.dim
    out = np.zeros((len(face_cell), 3 ** (dim - 1), dim))
    for fno in range(2 * dim):
        sel = np.nonzero(np.asarray(face_no) == fno)[0]
        if len(sel) == 0:
            continue
        pts, wts = face_reference_points(dim, fno)
        J = level.jacobians(pts)[np.asarray(face_cell)[sel]]  # (nf, nq, dim x, dim xi)
        d, side = divmod(fno, 2)
        tang = [a for a in range(dim) if a != d]
        if dim == 3:
            N = np.cross(J[..., tang[0]], J[..., tang[1]])
        else:
            t = J[..., tang[0]]
            N = np.stack([t[..., 1], -t[..., 0]], axis=-1)
        dn = np.einsum("fqi,fqi->fq", N, J[..., d])
        sgn = np.where((dn >= 0) == (side == 1), 1.0, -1.0)
        out[sel] = N * (sgn * wts[None, :])[..., None]
    return out


def boundary_faces(level: "LevelMesh", on_surface) -> tuple[np.ndarray, np.ndarray]:
    """(face_cell, face_no) of the cell faces whose centre x satisfies on_surface(x)
    (a vectorised predicate on (n, dim) points), in cell order."""
    dim = level.dim
    cells, nos = [], []
    for fno in range(2 * dim):
        d, side = divmod(fno, 2)
        c = np.full((1, dim), 0.5)
        c[0, d] = side
        x = level.map_points(c)[:, 0, :]
        hit = np.nonzero(on_surface(x))[0]
        cells.append(hit)
        nos.append(np.full(len(hit), fno))
    fc, fn = np.concatenate(cells), np.concatenate(nos)
    order = np.lexsort((fn, fc))
    return fc[order].astype(np.int32), fn[order].astype(np.int32)


def _lex(idx: tuple, shape: tuple) -> int:
    out, stride = 0, 1
    for i, n in zip(idx, shape):
        out += i * stride
        stride *= n
    return out


def box_level(dim: int, ncells: tuple, extent: tuple, origin: tuple | None = None,
              free_slip: bool = True, no_slip: bool = False, open_faces: tuple = (), degree: int = 2) -> LevelMesh:
    """Uniform axis-aligned box with lexicographic cells, component-blocked
    Q2 velocity numbering and lexicographic Q1 pressure numbering.

    ``free_slip``: no-normal-flux on every face (the normal component is a
    Dirichlet-zero line), as ``Tangential velocity boundary indicators`` gives
    on a box (VectorTools::compute_no_normal_flux_constraints on axis-aligned
    faces). ``no_slip``: every component is zero on every face, as ``Zero
    velocity boundary indicators`` on all faces gives. ``open_faces``: face
    numbers 2*d + side left without constraints (e.g. a free surface).
    ``degree``: velocity degree (2: Q2-Q1, 3: Q3-Q2 with Gauss-Lobatto velocity
    nodes)."""
    from . import fe
    origin = origin or (0.0,) * dim
    ncells = tuple(ncells)
    h = tuple(extent[d] / ncells[d] for d in range(dim))
    pd = degree - 1  # pressure degree
    nn = tuple(degree * n + 1 for n in ncells)  # velocity nodes per direction
    npn = tuple(pd * n + 1 for n in ncells)  # pressure nodes per direction
    n_nodes = int(np.prod(nn))
    n_pnodes = int(np.prod(npn))
    n_cells = int(np.prod(ncells))

    # cell multi-indices, x fastest
    cidx = np.stack(np.meshgrid(*[np.arange(n) for n in ncells], indexing="ij"), -1)
    cidx = cidx.transpose(*reversed(range(dim)), dim).reshape(-1, dim)  # x fastest
    loc = np.array(list(itertools.product(range(degree + 1), repeat=dim)))[:, ::-1]  # x fastest
    locp = np.array(list(itertools.product(range(pd + 1), repeat=dim)))[:, ::-1]

    strides = np.cumprod((1,) + nn[:-1])
    pstrides = np.cumprod((1,) + npn[:-1])
    node = ((degree * cidx[:, None, :] + loc[None, :, :]) * strides).sum(-1)  # (n_cells, (degree+1)^d)
    pnode = ((pd * cidx[:, None, :] + locp[None, :, :]) * pstrides).sum(-1)
    cell_dofs_u = np.concatenate([node + c * n_nodes for c in range(dim)], axis=1).astype(np.int32)
    cell_dofs_p = pnode.astype(np.int32)

    geom = np.zeros((n_cells, 2 * dim))
    for d in range(dim):
        geom[:, d] = origin[d] + cidx[:, d] * h[d]
        geom[:, dim + d] = h[d]

    # DoF positions: global node G along a direction lies in cell G // degree at
    # the local node G % degree (the last node closes the last cell)
    def coord(G, k, nodes):
        c = np.minimum(G // k, ncells[d_] - 1)
        return origin[d_] + (c + nodes[G - k * c]) * h[d_]

    vnodes, pnodes = fe.velocity_nodes(degree), fe.pressure_nodes(degree)
    nidx = np.stack(np.meshgrid(*[np.arange(n) for n in nn], indexing="ij"), -1)
    nidx = nidx.transpose(*reversed(range(dim)), dim).reshape(-1, dim)
    pidx = np.stack(np.meshgrid(*[np.arange(n) for n in npn], indexing="ij"), -1)
    pidx = pidx.transpose(*reversed(range(dim)), dim).reshape(-1, dim)
    pts_u, pts_p = [], []
    for d_ in range(dim):
        pts_u.append(coord(nidx[:, d_], degree, vnodes))
        pts_p.append(coord(pidx[:, d_], pd, pnodes))
    pts_u, pts_p = np.array(pts_u).T, np.array(pts_p).T

    lines = {}
    def face_nodes(d, side):
        return nidx[:, d] == (nn[d] - 1 if side else 0)

    closed = [f for f in range(2 * dim) if f not in tuple(open_faces)]
    if no_slip:
        on_bnd = np.zeros(n_nodes, bool)
        for f in closed:
            on_bnd |= face_nodes(f // 2, f % 2)
        for c in range(dim):
            for nd in np.nonzero(on_bnd)[0]:
                lines[int(nd + c * n_nodes)] = ([], 0.0)
    elif free_slip:
        for c in range(dim):
            on_face = np.zeros(n_nodes, bool)
            for f in closed:
                if f // 2 == c:
                    on_face |= face_nodes(c, f % 2)
            for nd in np.nonzero(on_face)[0]:
                lines[int(nd + c * n_nodes)] = ([], 0.0)
    cu = Constraints.from_dict(lines)

    return LevelMesh(dim=dim, n_cells=n_cells, n_u=dim * n_nodes, n_p=n_pnodes,
                     cell_dofs_u=cell_dofs_u, cell_dofs_p=cell_dofs_p, geom_kind=GEOM_BOX,
                     geometry=geom, constraints_u=cu, constraints_p=Constraints.empty(),
                     dof_points_u=np.tile(pts_u, (dim, 1)),
                     dof_component_u=np.repeat(np.arange(dim), n_nodes),
                     dof_points_p=pts_p, degree=degree)


def box_hierarchy(dim: int, n_fine: int, extent=None, n_coarse: int = 1,
                  free_slip: bool = True, no_slip: bool = False, open_faces: tuple = (),
                  degree: int = 2) -> list[LevelMesh]:
    """Global-coarsening hierarchy of uniform boxes: level l has n_coarse*2**l
    cells per direction, up to n_fine on the finest level."""
    extent = tuple(extent or (1.0,) * dim)
    levels = []
    n = n_coarse
    while n <= n_fine:
        levels.append(box_level(dim, (n,) * dim, extent, free_slip=free_slip, no_slip=no_slip,
                                open_faces=open_faces, degree=degree))
        n *= 2
    assert levels and n // 2 == n_fine, "n_fine must be n_coarse * 2**k"
    for l in range(1, len(levels)):
        nc = n_coarse * 2 ** l
        cidx = np.stack(np.meshgrid(*[np.arange(nc)] * dim, indexing="ij"), -1)
        cidx = cidx.transpose(*reversed(range(dim)), dim).reshape(-1, dim)
        par = cidx // 2
        pstr = np.cumprod((1,) + (nc // 2,) * (dim - 1))
        levels[l].parent = (par * pstr).sum(-1).astype(np.int32)
        levels[l].child_index = ((cidx % 2) << np.arange(dim)).sum(-1).astype(np.uint8)
    return levels


def permute_dofs(level: LevelMesh, seed: int) -> tuple[LevelMesh, np.ndarray, np.ndarray]:
    """Return a copy with randomly renumbered DoFs (tests that the library does not
    depend on the caller's numbering). Returns (mesh, perm_u, perm_p) where
    new_index = perm[old_index]."""
    rng = np.random.default_rng(seed)
    pu = rng.permutation(level.n_u).astype(np.int32)
    pp = rng.permutation(level.n_p).astype(np.int32)

    def remap(c: Constraints, perm):
        lines = {}
        for i, r in enumerate(c.rows):
            a, b = c.ptr[i], c.ptr[i + 1]
            lines[int(perm[r])] = ([(int(perm[cc]), float(w)) for cc, w in
                                    zip(c.cols[a:b], c.weights[a:b])], float(c.inhom[i]))
        return Constraints.from_dict(lines)

    inv_u = np.argsort(pu)
    inv_p = np.argsort(pp)
    out = dataclasses.replace(
        level, cell_dofs_u=pu[level.cell_dofs_u].astype(np.int32),
        cell_dofs_p=pp[level.cell_dofs_p].astype(np.int32),
        constraints_u=remap(level.constraints_u, pu), constraints_p=remap(level.constraints_p, pp),
        dof_points_u=level.dof_points_u[inv_u] if level.dof_points_u is not None else None,
        dof_component_u=level.dof_component_u[inv_u] if level.dof_component_u is not None else None,
        dof_points_p=level.dof_points_p[inv_p] if level.dof_points_p is not None else None)
    return out, pu, pp


def to_q2_geometry(level: LevelMesh, distortion=None) -> LevelMesh:
    """Same level with GEOM_Q2 cell geometry (3^dim support points per cell),
    optionally moved by ``distortion(x) -> dx`` (applied pointwise, so shared
    points stay shared)."""
    X = level.q2_support_points().copy()
    if distortion is not None:
        flat = X.reshape(-1, level.dim)
        X = (flat + distortion(flat)).reshape(X.shape)
    return dataclasses.replace(level, geom_kind=GEOM_Q2, geometry=X.reshape(level.n_cells, -1))


def to_table_geometry(level: LevelMesh, jacobians: np.ndarray | None = None) -> LevelMesh:
    """Same level with GEOM_TABLE cell geometry: per cell and QGauss(degree+1)
    point the inverse Jacobian (d xi_d / d x_e at [d*dim+e]) and |det J|.
    ``jacobians`` (n_cells, (degree+1)**dim, dim, dim) [x-component, xi-direction]
    are the caller's mapping at the Gauss points; by default the level's own mapping."""
    from . import fe
    gp = fe.tensor_points(level.dim, fe.gauss(level.degree + 1)[0])
    J = level.jacobians(gp) if jacobians is None else np.asarray(jacobians, float)
    inv = np.linalg.inv(J)
    det = np.abs(np.linalg.det(J))
    d = level.dim
    table = np.concatenate([inv.reshape(level.n_cells, len(gp), d * d), det[..., None]], axis=-1)
    return dataclasses.replace(level, geom_kind=GEOM_TABLE, geometry=table.reshape(level.n_cells, -1))


def smooth_distortion(amplitude: float = 0.03):
    """A displacement that vanishes on the boundary of the unit box."""
    def f(x):
        b = np.prod(np.sin(np.pi * x), axis=1)
        d = np.zeros_like(x)
        for k in range(x.shape[1]):
            d[:, k] = amplitude * b * np.cos(np.pi * (k + 1) * x[:, (k + 1) % x.shape[1]])
        return d
    return f
