"""ctypes front end of libgb_gmg.so (the C ABI in include/gb_gmg.h).

:class:`StokesMatrixFreeGPU` mirrors ASPECT's StokesMatrixFreeHandler
(include/aspect/simulator/solver/stokes_matrix_free.h:47-98) and
StokesSolver::Interface::solve (include/aspect/simulator/solver/interface.h:90-94):
``setup_dofs`` / ``assemble`` / ``build_preconditioner`` / ``solve``, with the
same argument meaning (scaled pressure p/s in the solve vectors) and the same
error behaviour (a failed solve raises, like SolverControl::NoConvergence).

The CUDA library is required: importing the front end without a built
libgb_gmg.so, or using it without a CUDA device, raises; there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgb_gmg.so")

OP_STOKES, OP_A, OP_BT, OP_MASS = 0, 1, 2, 3
FP64, FP32 = 0, 1
GMRES, GMRES_IR, IDR = 0, 1, 2
VISC_DGQ0, VISC_DGQ1, VISC_NONE = 0, 1, 2
COARSE_CHEBYSHEV, COARSE_DENSE_FP64 = 0, 1

STATUS = {0: "OK", 1: "INVALID_ARGUMENT", 2: "NOT_READY", 3: "CUDA_ERROR", 4: "NO_CONVERGENCE",
          5: "BREAKDOWN", 6: "NAN_DETECTED", 7: "OUT_OF_MEMORY", 8: "EXCEEDS_STATIC_SCRATCH"}


class GmgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class NoConvergence(GmgError):
    pass


class Options(ctypes.Structure):
    _fields_ = [("verbose", ctypes.c_int), ("smoother_degree", ctypes.c_int),
                ("smoothing_range", ctypes.c_double), ("eig_cg_iterations", ctypes.c_int),
                ("coarse_degree", ctypes.c_int), ("coarse_range", ctypes.c_double),
                ("coarse_eig_cg_iterations", ctypes.c_int), ("schur_smoothing_steps", ctypes.c_int),
                ("force_indexed_layout", ctypes.c_int), ("coarse_solver", ctypes.c_int),
                ("fused_a_min_cells", ctypes.c_int), ("dense_mass_cycle_nodes", ctypes.c_int),
                ("dense_a_cycle_dofs", ctypes.c_int), ("fused_small_smoother", ctypes.c_int)]


class SolveParams(ctypes.Structure):
    _fields_ = [("linear_solver_tolerance", ctypes.c_double), ("absolute_tolerance", ctypes.c_double),
                ("n_cheap_steps", ctypes.c_int), ("n_expensive_steps", ctypes.c_int),
                ("restart", ctypes.c_int), ("tol_A", ctypes.c_double), ("tol_S", ctypes.c_double),
                ("mg_precision", ctypes.c_int), ("krylov", ctypes.c_int),
                ("ir_inner_tolerance", ctypes.c_double), ("idr_s", ctypes.c_int),
                ("solve_newton_system", ctypes.c_int), ("orthogonalization", ctypes.c_int)]


class NewtonTerms(ctypes.Structure):
    _fields_ = [("enable_newton_derivatives", ctypes.c_int), ("symmetrize_newton_system", ctypes.c_int),
                ("average_newton_factors", ctypes.c_int), ("enable_prescribed_dilation", ctypes.c_int),
                ("strain_rate", ctypes.c_void_p), ("newton_factor_wrt_strain_rate", ctypes.c_void_p),
                ("newton_factor_wrt_pressure", ctypes.c_void_p), ("dilation_lhs", ctypes.c_void_p),
                ("dilation_derivative_wrt_strain_rate", ctypes.c_void_p),
                ("dilation_derivative_wrt_pressure", ctypes.c_void_p)]


class Outputs(ctypes.Structure):
    _fields_ = [("initial_nonlinear_residual", ctypes.c_double), ("final_linear_residual", ctypes.c_double),
                ("solver_tolerance", ctypes.c_double), ("cheap_iterations", ctypes.c_int),
                ("expensive_iterations", ctypes.c_int), ("A_preconditioner_applications", ctypes.c_int),
                ("S_preconditioner_applications", ctypes.c_int), ("fp64_stokes_applications", ctypes.c_int),
                ("status", ctypes.c_int), ("solve_seconds", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


EXPORTS = ["gb_gmg_default_options", "gb_gmg_default_solve_params", "gb_gmg_create", "gb_gmg_destroy",
           "gb_gmg_last_error", "gb_gmg_set_level_mesh", "gb_gmg_set_level_constraints", "gb_gmg_set_transfer",
           "gb_gmg_finalize_setup", "gb_gmg_set_viscosity", "gb_gmg_build_preconditioner", "gb_gmg_vmult",
           "gb_gmg_vmult_device", "gb_gmg_get_diagonal_inverse", "gb_gmg_get_eigenvalues",
           "gb_gmg_set_eigenvalues", "gb_gmg_transfer", "gb_gmg_vcycle", "gb_gmg_block_preconditioner",
           "gb_gmg_solve", "gb_gmg_solve_device", "gb_gmg_adjoint_gradient", "gb_gmg_memory_consumption",
           "gb_gmg_kernel_launches", "gb_gmg_time_operation", "gb_gmg_ablock_apply_lattice_noalloc",
           "gb_gmg_update_viscosity", "gb_gmg_correct_stokes_rhs", "gb_gmg_set_newton_terms",
           "gb_gmg_assemble_rhs", "gb_gmg_set_free_surface"]

TIME_STOKES_VMULT, TIME_A_VMULT, TIME_MASS_VMULT = 0, 1, 2
TIME_STOKES_PRECONDITIONER, TIME_A_PRECONDITIONER, TIME_S_PRECONDITIONER = 3, 4, 5
TIME_A_CELL_PASS = 6
TIME_STOKES_CELL_PASS = 7

_lib = None


def load_library(path: str = LIB_PATH):
    """Load libgb_gmg.so; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m aspect_gb300.build` "
                          "(the GMG Stokes solver has no CPU fallback)")
    L = ctypes.CDLL(path)
    vp, dp, ip, i64 = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64
    L.gb_gmg_create.argtypes = [ctypes.POINTER(Options), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                ctypes.POINTER(ctypes.c_void_p)]
    L.gb_gmg_destroy.argtypes = [vp]
    L.gb_gmg_destroy.restype = None
    L.gb_gmg_last_error.argtypes = [vp]
    L.gb_gmg_last_error.restype = ctypes.c_char_p
    L.gb_gmg_default_options.argtypes = [ctypes.POINTER(Options)]
    L.gb_gmg_default_options.restype = None
    L.gb_gmg_default_solve_params.argtypes = [ctypes.POINTER(SolveParams)]
    L.gb_gmg_default_solve_params.restype = None
    L.gb_gmg_set_level_mesh.argtypes = [vp, ctypes.c_int, i64, ip, ip, ctypes.c_int, dp, i64, i64]
    L.gb_gmg_set_level_constraints.argtypes = [vp, ctypes.c_int, ctypes.c_int, i64, ip, ip, ip, dp, dp]
    L.gb_gmg_set_transfer.argtypes = [vp, ctypes.c_int, ip, ip]
    L.gb_gmg_finalize_setup.argtypes = [vp]
    L.gb_gmg_set_viscosity.argtypes = [vp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int]
    L.gb_gmg_build_preconditioner.argtypes = [vp]
    L.gb_gmg_update_viscosity.argtypes = [vp, dp, ctypes.c_int]
    L.gb_gmg_set_newton_terms.argtypes = [vp, ctypes.POINTER(NewtonTerms)]
    L.gb_gmg_vmult.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp]
    L.gb_gmg_correct_stokes_rhs.argtypes = [vp, dp, dp]
    L.gb_gmg_assemble_rhs.argtypes = [vp, dp, dp]
    L.gb_gmg_set_free_surface.argtypes = [vp, ctypes.c_int64, vp, vp, vp, vp]
    L.gb_gmg_vmult_device.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp, dp]
    L.gb_gmg_get_diagonal_inverse.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    L.gb_gmg_get_eigenvalues.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    L.gb_gmg_set_eigenvalues.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp]
    L.gb_gmg_transfer.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, dp]
    L.gb_gmg_vcycle.argtypes = [vp, ctypes.c_int, ctypes.c_int, dp, dp]
    L.gb_gmg_block_preconditioner.argtypes = [vp, ctypes.c_int, dp, dp]
    L.gb_gmg_solve.argtypes = [vp, dp, dp, ctypes.POINTER(SolveParams), ctypes.POINTER(Outputs)]
    L.gb_gmg_solve_device.argtypes = [vp, dp, dp, ctypes.POINTER(SolveParams), ctypes.POINTER(Outputs)]
    L.gb_gmg_adjoint_gradient.argtypes = [vp, dp, dp, dp]
    L.gb_gmg_memory_consumption.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
    L.gb_gmg_kernel_launches.argtypes = [vp]
    L.gb_gmg_kernel_launches.restype = ctypes.c_int64
    L.gb_gmg_time_operation.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_double)]
    L.gb_gmg_ablock_apply_lattice_noalloc.argtypes = [ctypes.c_int, vp, vp, ctypes.c_uint32, ctypes.c_int, vp, vp,
                                                      vp, vp]
    _lib = L
    return L


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _at_least(a: np.ndarray, n: int, what: str) -> np.ndarray:
    """The library reads (or writes) n entries through the array's pointer: a
    shorter array is rejected with its INVALID_ARGUMENT status before the call."""
    if a.size < n:
        raise GmgError(1, f"{what} has {a.size} entries; the library uses {n}")
    return a


def _assign_fields(struct: ctypes.Structure, values: dict, what: str) -> None:
    """Sets the named fields of a ctypes mirror of a header struct; a name that
    is not a field raises instead of becoming a plain (ignored) attribute."""
    names = [f for f, _ in type(struct)._fields_]
    for k, v in values.items():
        if k not in names:
            raise TypeError(f"unknown {what} {k!r}; known: {', '.join(names)}")
        setattr(struct, k, v)


def default_solve_params(**kw) -> SolveParams:
    p = SolveParams()
    load_library().gb_gmg_default_solve_params(ctypes.byref(p))
    _assign_fields(p, kw, "solve parameter")
    return p


class StokesMatrixFreeGPU:
    """GPU matrix-free GMG Stokes solver behind the C ABI; name() = "GMG-GB300"."""

    def __init__(self, dim: int, n_levels: int, options: dict | None = None, degree: int = 2):
        """degree: the velocity degree ("Stokes velocity polynomial degree"), 2 (Q2-Q1)
        or 3 (Q3-Q2)."""
        self.L = load_library()
        opt = Options()
        self.L.gb_gmg_default_options(ctypes.byref(opt))
        _assign_fields(opt, options or {}, "option")
        h = ctypes.c_void_p()
        rc = self.L.gb_gmg_create(ctypes.byref(opt), dim, degree, n_levels, ctypes.byref(h))
        if rc != 0:
            raise GmgError(rc, "gb_gmg_create failed")
        self.h = h
        self.dim = dim
        self.degree = degree
        self.n_levels = n_levels
        self.levels = None

    @staticmethod
    def name() -> str:
        return "GMG-GB300"

    def __del__(self):
        try:
            if self.h:
                self.L.gb_gmg_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def _chk(self, rc):
        if rc != 0:
            msg = self.L.gb_gmg_last_error(self.h).decode()
            raise (NoConvergence if rc == 4 else GmgError)(rc, msg)

    # ---------------------------------------------------------------- set-up
    def setup_dofs(self, levels):
        """Hand over the level meshes, constraints and parent/child data."""
        self.levels = levels
        keep = []
        d, k = self.dim, self.degree
        for l, m in enumerate(levels):
            cdu, cdp, g = _i(m.cell_dofs_u), _i(m.cell_dofs_p), _d(m.geometry)
            # the library reads these many entries (gb_gmg_set_level_mesh)
            n_geom = {0: 2 * d, 1: 3 ** d * d, 2: (k + 1) ** d * (d * d + 1)}[m.geom_kind]
            if (cdu.size != m.n_cells * d * (k + 1) ** d or cdp.size != m.n_cells * k ** d
                    or g.size != m.n_cells * n_geom):
                raise ValueError(f"level {l}: cell DoF or geometry arrays do not match degree {k}")
            keep += [cdu, cdp, g]
            self._chk(self.L.gb_gmg_set_level_mesh(self.h, l, m.n_cells, _p(cdu), _p(cdp), m.geom_kind, _p(g),
                                                   m.n_u, m.n_p))
            for block, c in enumerate([m.constraints_u, m.constraints_p]):
                arrs = [_i(c.rows), _i(c.ptr), _i(c.cols), _d(c.weights), _d(c.inhom)]
                keep += arrs
                self._chk(self.L.gb_gmg_set_level_constraints(self.h, l, block, c.n_lines, *[_p(a) for a in arrs]))
            if l > 0:
                par = _i(m.parent)
                ch = np.ascontiguousarray(m.child_index, dtype=np.uint8)
                keep += [par, ch]
                self._chk(self.L.gb_gmg_set_transfer(self.h, l, _p(par), _p(ch)))
        self._chk(self.L.gb_gmg_finalize_setup(self.h))

    def assemble(self, eta, projection: int, pressure_scaling: float, compressible: int = 0):
        """evaluate_material_model: finest-level viscosity (per cell or per quadrature point)."""
        eta = _at_least(_d(eta), self.levels[-1].n_cells, "viscosity")
        n_per_cell = eta.size // self.levels[-1].n_cells
        self._chk(self.L.gb_gmg_set_viscosity(self.h, _p(eta), n_per_cell, projection,
                                              ctypes.c_double(pressure_scaling), compressible))

    def update_viscosity(self, eta):
        """New viscosity for the operators; keeps the last-built preconditioner."""
        eta = _at_least(_d(eta), self.levels[-1].n_cells, "viscosity")
        self._chk(self.L.gb_gmg_update_viscosity(self.h, _p(eta), eta.size // self.levels[-1].n_cells))

    def set_newton_terms(self, newton=False, symmetrize=False, average=False, dilation=False, strain_rate=None,
                         d_eta_d_strain_rate=None, d_eta_d_pressure=None, dilation_lhs=None,
                         d_dilation_d_strain_rate=None, d_dilation_d_pressure=None):
        """OperatorCellData's Newton / prescribed-dilation tables of the outer Stokes
        operator (per finest cell and quadrature point); all flags False clears them."""
        if not (newton or dilation):
            self._chk(self.L.gb_gmg_set_newton_terms(self.h, None))
            return
        arrs = [None if a is None else _d(a) for a in (strain_rate, d_eta_d_strain_rate, d_eta_d_pressure,
                                                          dilation_lhs, d_dilation_d_strain_rate, d_dilation_d_pressure)]
        t = NewtonTerms(int(newton), int(symmetrize), int(average), int(dilation),
                        *[None if a is None else a.ctypes.data for a in arrs])
        self._chk(self.L.gb_gmg_set_newton_terms(self.h, ctypes.byref(t)))

    def set_free_surface(self, face_cell=None, face_no=None, stabilization=None, normal_jxw=None):
        """Free-surface stabilisation faces of the outer Stokes operator
        (StokesOperator::local_apply_boundary_face): face_cell / face_no per face,
        stabilization (n_faces, 3**(dim-1), dim) = rho dt theta |g| g_hat at the
        face points, normal_jxw the same shape or None (from the level geometry).
        No arguments: the term is removed."""
        if face_cell is None or len(face_cell) == 0:
            self._chk(self.L.gb_gmg_set_free_surface(self.h, 0, None, None, None, None))
            return
        fc = np.ascontiguousarray(face_cell, dtype=np.int32)
        fn = np.ascontiguousarray(face_no, dtype=np.int32)
        st = _d(stabilization)
        nj = None if normal_jxw is None else _d(normal_jxw)
        self._chk(self.L.gb_gmg_set_free_surface(self.h, len(fc), _p(fc), _p(fn), _p(st),
                                                 None if nj is None else _p(nj)))

    def build_preconditioner(self):
        """Diagonals and Chebyshev eigenvalue estimates of every level; the FP64
        levels are built on their first use (gb_gmg_build_preconditioner)."""
        self._chk(self.L.gb_gmg_build_preconditioner(self.h))

    # ---------------------------------------------------------------- solve
    def solve(self, rhs, x0=None, **params):
        """Returns (solution [u; p/s], outputs dict). Raises NoConvergence on failure."""
        rhs = _d(rhs)
        sol = _d(np.zeros_like(rhs) if x0 is None else x0).copy()
        if self.levels is not None:
            _at_least(rhs, self._n_top(), "rhs")
            _at_least(sol, self._n_top(), "x0")
        prm = default_solve_params(**params)
        out = Outputs()
        self._chk(self.L.gb_gmg_solve(self.h, _p(rhs), _p(sol), ctypes.byref(prm), ctypes.byref(out)))
        return sol, out.as_dict()

    def solve_device(self, d_rhs_ptr: int, d_sol_ptr: int, **params) -> dict:
        prm = default_solve_params(**params)
        out = Outputs()
        self._chk(self.L.gb_gmg_solve_device(self.h, ctypes.c_void_p(d_rhs_ptr), ctypes.c_void_p(d_sol_ptr),
                                             ctypes.byref(prm), ctypes.byref(out)))
        return out.as_dict()

    # ---------------------------------------------------------------- pieces
    def vmult(self, op: int, level: int, src, precision: int = FP64):
        m = self.levels[level]
        n_out = m.n_u + m.n_p if op == OP_STOKES else (m.n_p if op == OP_MASS else m.n_u)
        n_in = m.n_u + m.n_p if op == OP_STOKES else (m.n_u if op == OP_A else m.n_p)
        src = _at_least(_d(src), n_in, "src")
        out = np.zeros(n_out)
        self._chk(self.L.gb_gmg_vmult(self.h, op, level, precision, _p(src), _p(out)))
        return out

    def correct_stokes_rhs(self, u0, rhs):
        """rhs - K u0 (plain reads of u0, which holds the inhomogeneous constraint
        values), as StokesMatrixFreeHandler::correct_stokes_rhs; returns a new array."""
        u0 = _at_least(_d(u0), self._n_top(), "u0")
        out = _at_least(_d(rhs).copy(), self._n_top(), "rhs")
        self._chk(self.L.gb_gmg_correct_stokes_rhs(self.h, _p(u0), _p(out)))
        return out

    def assemble_rhs(self, force_q):
        """Body-force right-hand side int f . phi_u of the finest level on the device,
        condensed with the velocity constraints; force_q: (n_cells, 3**dim, dim)."""
        f = _d(force_q)
        if self.degree == 2:  # other degrees: the library's own rejection
            _at_least(f, self.levels[-1].n_cells * 3 ** self.dim * self.dim, "force_q")
        out = np.zeros(self.levels[-1].n_u + self.levels[-1].n_p)
        self._chk(self.L.gb_gmg_assemble_rhs(self.h, _p(f), _p(out)))
        return out

    def vmult_device(self, d_src: int, d_dst: int, precision: int = FP64):
        self._chk(self.L.gb_gmg_vmult_device(self.h, OP_STOKES, precision, ctypes.c_void_p(d_src),
                                             ctypes.c_void_p(d_dst)))

    def diagonal_inverse(self, level: int, block: int, precision: int = FP64):
        m = self.levels[level]
        out = np.zeros(m.n_u if block == 0 else m.n_p)
        self._chk(self.L.gb_gmg_get_diagonal_inverse(self.h, level, block, precision, _p(out)))
        return out

    def eigenvalues(self, level: int, block: int, precision: int = FP64):
        out = np.zeros(2)
        self._chk(self.L.gb_gmg_get_eigenvalues(self.h, level, block, precision, _p(out)))
        return out

    def set_eigenvalues(self, level: int, block: int, precision: int, minmax):
        v = _at_least(_d(minmax), 2, "minmax")
        self._chk(self.L.gb_gmg_set_eigenvalues(self.h, level, block, precision, _p(v)))

    def transfer(self, fine_level: int, block: int, restrict: bool, src, precision: int = FP64):
        tgt = self.levels[fine_level - 1 if restrict else fine_level]
        out = np.zeros(tgt.n_u if block == 0 else tgt.n_p)
        src = _d(src)
        if 1 <= fine_level < len(self.levels):  # other levels: the library's own rejection
            srcl = self.levels[fine_level if restrict else fine_level - 1]
            _at_least(src, srcl.n_u if block == 0 else srcl.n_p, "src")
        self._chk(self.L.gb_gmg_transfer(self.h, fine_level, block, precision, int(restrict), _p(src), _p(out)))
        return out

    def vcycle(self, block: int, src, precision: int = FP64):
        src = _d(src)
        if block in (0, 1):
            _at_least(src, self.levels[-1].n_u if block == 0 else self.levels[-1].n_p, "src")
        out = np.zeros_like(src)
        self._chk(self.L.gb_gmg_vcycle(self.h, block, precision, _p(src), _p(out)))
        return out

    def block_preconditioner(self, src, precision: int = FP64):
        src = _at_least(_d(src), self._n_top(), "src")
        out = np.zeros_like(src)
        self._chk(self.L.gb_gmg_block_preconditioner(self.h, precision, _p(src), _p(out)))
        return out

    def adjoint_gradient(self, u, lam):
        u = _at_least(_d(u), self.levels[-1].n_u, "u")
        lam = _at_least(_d(lam), self.levels[-1].n_u, "lam")
        out = np.zeros(self.levels[-1].n_cells)
        self._chk(self.L.gb_gmg_adjoint_gradient(self.h, _p(u), _p(lam), _p(out)))
        return out

    def memory_consumption(self) -> int:
        b = ctypes.c_size_t()
        self._chk(self.L.gb_gmg_memory_consumption(self.h, ctypes.byref(b)))
        return b.value

    def time_operation(self, what: int, precision: int = FP64, repeats: int = 10) -> float:
        """Mean device seconds of one call (stokes_vmult, A/S/stokes preconditioner, ...)."""
        sec = ctypes.c_double()
        self._chk(self.L.gb_gmg_time_operation(self.h, what, precision, repeats, ctypes.byref(sec)))
        return sec.value

    def _n_top(self) -> int:
        return self.levels[-1].n_u + self.levels[-1].n_p

    def kernel_launches(self) -> int:
        return int(self.L.gb_gmg_kernel_launches(self.h))


def from_problem(problem, options: dict | None = None, build: bool = True) -> StokesMatrixFreeGPU:
    """Set up a solver for a :class:`aspect_gb300.problems.StokesProblem`."""
    s = StokesMatrixFreeGPU(problem.levels[0].dim, len(problem.levels), options,
                            degree=getattr(problem.levels[0], "degree", 2))
    s.setup_dofs(problem.levels)
    s.assemble(problem.eta, problem.projection, problem.pressure_scaling)
    if build:
        s.build_preconditioner()
    return s
