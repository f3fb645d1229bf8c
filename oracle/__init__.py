"""ctypes front end of the CPU oracle (``gmg_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``, always as the checker. The product
library never imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_up = ctypes.POINTER(ctypes.c_ubyte)


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "gmg_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE])
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int, ctypes.c_int]
        L.orc_create_degree.restype = ctypes.c_void_p
        L.orc_create_degree.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_last_error.argtypes = [ctypes.c_void_p]
        for name in ["orc_set_level_mesh", "orc_set_level_constraints", "orc_set_transfer",
                     "orc_finalize", "orc_set_viscosity", "orc_get_level_viscosity",
                     "orc_build_preconditioner", "orc_vmult", "orc_get_diagonal", "orc_transfer",
                     "orc_estimate_eigenvalues", "orc_get_eigenvalues", "orc_set_eigenvalues",
                     "orc_vcycle", "orc_block_preconditioner", "orc_solve", "orc_adjoint_gradient",
                     "orc_set_fast", "orc_set_newton", "orc_set_free_surface"]:
            getattr(L, name).restype = ctypes.c_int
        _lib = L
    return _lib


def set_fast(on: bool) -> None:
    """Process-wide switch of the oracle library: True selects the sum-factorised
    cell operators and parallel reductions used to time the CPU baseline; False
    (the default) the plain quadrature loops the parity tests check against."""
    lib().orc_set_fast(int(bool(on)))


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a, t):
    return a.ctypes.data_as(t)


class Oracle:
    """CPU restatement of the solver for one level hierarchy (list of LevelMesh)."""

    def __init__(self, levels, n_threads: int = 0):
        self.L = lib()
        if n_threads:
            self.L.orc_set_num_threads(int(n_threads))
        self.levels = levels
        self.dim = levels[0].dim
        self.degree = getattr(levels[0], "degree", 2)  # velocity degree of the level meshes
        self.h = ctypes.c_void_p(self.L.orc_create_degree(self.dim, self.degree, len(levels)))
        for l, m in enumerate(levels):
            cdu, cdp, g = _i(m.cell_dofs_u), _i(m.cell_dofs_p), _d(m.geometry)
            self._chk(self.L.orc_set_level_mesh(self.h, l, m.n_cells, _ptr(cdu, _ip), _ptr(cdp, _ip),
                                                m.geom_kind, _ptr(g, _dp), m.n_u, m.n_p))
            for block, c in enumerate([m.constraints_u, m.constraints_p]):
                rows, ptr, cols = _i(c.rows), _i(c.ptr), _i(c.cols)
                w, b = _d(c.weights), _d(c.inhom)
                self._chk(self.L.orc_set_level_constraints(
                    self.h, l, block, c.n_lines, _ptr(rows, _ip), _ptr(ptr, _ip), _ptr(cols, _ip),
                    _ptr(w, _dp), _ptr(b, _dp)))
            if l > 0:
                par = _i(m.parent)
                ch = np.ascontiguousarray(m.child_index, dtype=np.uint8)
                self._chk(self.L.orc_set_transfer(self.h, l, _ptr(par, _ip), _ptr(ch, _up)))
        self._chk(self.L.orc_finalize(self.h))

    def __del__(self):
        try:
            self.L.orc_destroy(self.h)
        except Exception:
            pass

    def _chk(self, rc):
        if rc != 0:
            raise RuntimeError("oracle: " + self.L.orc_last_error(self.h).decode())

    @property
    def fine(self):
        return self.levels[-1]

    def set_viscosity(self, eta, projection: int, pressure_scaling: float, compressible: int = 0,
                      mg_finest_projected: bool = False):
        """mg_finest_projected (per-point eta, projection 0): the multigrid levels,
        the finest included, use the cellwise projection while the outer operators
        keep the per-point values, as the reference does without averaging."""
        eta = _d(eta)
        n_per_cell = eta.size // self.fine.n_cells
        self._chk(self.L.orc_set_viscosity(self.h, _ptr(eta, _dp), n_per_cell, projection,
                                           ctypes.c_double(pressure_scaling), compressible,
                                           int(mg_finest_projected)))

    def level_viscosity(self, level: int) -> np.ndarray:
        m = self.levels[level]
        out = np.zeros(m.n_cells * 27)
        n = ctypes.c_int()
        self._chk(self.L.orc_get_level_viscosity(self.h, level, _ptr(out, _dp), ctypes.byref(n)))
        return out[: m.n_cells * n.value].reshape(m.n_cells, n.value)

    def build_preconditioner(self, mg_float: bool):
        self._chk(self.L.orc_build_preconditioner(self.h, int(mg_float)))

    def vmult(self, op: int, level: int, src, use_float: bool = False) -> np.ndarray:
        m = self.levels[level]
        n_out = m.n_u + m.n_p if op == 0 else (m.n_p if op == 3 else m.n_u)
        src = _d(src)
        out = np.zeros(n_out)
        self._chk(self.L.orc_vmult(self.h, op, level, int(use_float), _ptr(src, _dp), _ptr(out, _dp)))
        return out

    def diagonal_inverse(self, level: int, block: int) -> np.ndarray:
        m = self.levels[level]
        out = np.zeros(m.n_u if block == 0 else m.n_p)
        self._chk(self.L.orc_get_diagonal(self.h, level, block, _ptr(out, _dp)))
        return out

    def transfer(self, fine_level: int, block: int, restrict: bool, src) -> np.ndarray:
        tgt = self.levels[fine_level - 1 if restrict else fine_level]
        out = np.zeros(tgt.n_u if block == 0 else tgt.n_p)
        src = _d(src)
        self._chk(self.L.orc_transfer(self.h, fine_level, block, int(restrict), _ptr(src, _dp),
                                      _ptr(out, _dp)))
        return out

    def estimate_eigenvalues(self):
        self._chk(self.L.orc_estimate_eigenvalues(self.h))

    def eigenvalues(self, level: int, block: int) -> np.ndarray:
        out = np.zeros(2)
        self._chk(self.L.orc_get_eigenvalues(self.h, level, block, _ptr(out, _dp)))
        return out

    def set_eigenvalues(self, level: int, block: int, minmax):
        v = _d(minmax)
        self._chk(self.L.orc_set_eigenvalues(self.h, level, block, _ptr(v, _dp)))

    def vcycle(self, block: int, src) -> np.ndarray:
        src = _d(src)
        out = np.zeros_like(src)
        self._chk(self.L.orc_vcycle(self.h, block, _ptr(src, _dp), _ptr(out, _dp)))
        return out

    def block_preconditioner(self, src, expensive: bool = False) -> np.ndarray:
        src = _d(src)
        out = np.zeros_like(src)
        self._chk(self.L.orc_block_preconditioner(self.h, int(expensive), _ptr(src, _dp), _ptr(out, _dp)))
        return out

    def set_newton_terms(self, newton=False, symmetrize=False, average=False, dilation=False, strain_rate=None,
                         d_eta_d_strain_rate=None, d_eta_d_pressure=None, dilation_lhs=None,
                         d_dilation_d_strain_rate=None, d_dilation_d_pressure=None):
        flags = int(newton) | int(symmetrize) << 1 | int(average) << 2 | int(dilation) << 3
        arrs = [None if a is None else _d(a) for a in (strain_rate, d_eta_d_strain_rate, d_eta_d_pressure,
                                                          dilation_lhs, d_dilation_d_strain_rate, d_dilation_d_pressure)]
        self._chk(self.L.orc_set_newton(self.h, flags, *[None if a is None else _ptr(a, _dp) for a in arrs]))

    def set_free_surface(self, face_cell=None, face_no=None, stabilization=None, normal_jxw=None):
        """Free-surface faces of the outer Stokes operator (finest level): T per
        face point (n_faces, 3**(dim-1), dim) and the outward normal times JxW
        (same shape; None: from the level geometry by the harness). No arguments:
        the term is removed."""
        if face_cell is None or len(face_cell) == 0:
            self._chk(self.L.orc_set_free_surface(self.h, 0, None, None, None))
            return
        from aspect_gb300 import mesh
        fc = np.ascontiguousarray(face_cell, dtype=np.int32)
        fn = np.ascontiguousarray(face_no, dtype=np.int32)
        nj = mesh.face_normal_jxw(self.fine, fc, fn) if normal_jxw is None else _d(normal_jxw)
        tab = _d(np.concatenate([_d(stabilization), _d(nj)], axis=-1))
        self._chk(self.L.orc_set_free_surface(self.h, len(fc), _ptr(fc, ctypes.POINTER(ctypes.c_int)),
                                              _ptr(fn, ctypes.POINTER(ctypes.c_int)), _ptr(tab, _dp)))

    def adjoint_gradient(self, u, lam) -> np.ndarray:
        u, lam = _d(u), _d(lam)
        out = np.zeros(self.fine.n_cells)
        self._chk(self.L.orc_adjoint_gradient(self.h, _ptr(u, _dp), _ptr(lam, _dp), _ptr(out, _dp)))
        return out

    def solve(self, rhs, x0=None, tol_rel=1e-7, abs_tol=0.0, n_cheap=1000, n_expensive=1000,
              restart=100, tol_A=1e-2, tol_S=1e-6, krylov=0, idr_s=2):
        rhs = _d(rhs)
        sol = _d(np.zeros_like(rhs) if x0 is None else x0).copy()
        params = _d([tol_rel, abs_tol, n_cheap, n_expensive, restart, tol_A, tol_S, krylov, idr_s])
        out = np.zeros(8)
        self._chk(self.L.orc_solve(self.h, _ptr(params, _dp), _ptr(rhs, _dp), _ptr(sol, _dp),
                                   _ptr(out, _dp)))
        info = dict(initial_nonlinear_residual=out[0], final_linear_residual=out[1],
                    solver_tolerance=out[2], cheap_iterations=int(out[3]),
                    expensive_iterations=int(out[4]), A_preconditioner_applications=int(out[5]),
                    S_preconditioner_applications=int(out[6]), status=int(out[7]))
        return sol, info
