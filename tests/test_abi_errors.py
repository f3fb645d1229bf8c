"""Host-side behaviour of the C ABI that needs no GPU: argument checks that
return status codes before any CUDA call, the reference's parameter defaults
(source/simulator/parameters.cc:491-585), the allocation-free entry point's size
limit, and -- on a host without a GPU -- a handle that refuses to exist (there
is no CPU fallback)."""
import ctypes

import numpy as np
import pytest

from aspect_gb300 import gmg

OK, INVALID, NOT_READY, CUDA_ERROR, EXCEEDS = 0, 1, 2, 3, 8


@pytest.fixture(scope="module")
def L():
    return gmg.load_library()


def test_solve_parameter_defaults_follow_the_reference(L):
    p = gmg.default_solve_params()
    assert p.linear_solver_tolerance == 1e-7        # "Linear solver tolerance"
    assert p.n_cheap_steps == 1000                  # "Number of cheap Stokes solver steps"
    assert p.n_expensive_steps == 1000              # "Maximum number of expensive Stokes solver steps"
    assert p.restart == 100                         # "GMRES solver restart length" (Stokes)
    assert p.tol_A == 1e-2 and p.tol_S == 1e-6      # "Linear solver A / S block tolerance"
    assert p.krylov == gmg.GMRES and p.idr_s == 2   # "Krylov method for cheap solver steps", "IDR(s) parameter"
    assert p.absolute_tolerance == 0.0


def test_misspelled_parameter_names_are_rejected(L):
    """The Python front end sets only fields the header declares: a misspelled
    solve parameter or option raises (ctypes would otherwise keep it as a plain
    attribute and the library would never see it); known names still set."""
    with pytest.raises(TypeError, match="linear_solver_tolerence"):
        gmg.default_solve_params(linear_solver_tolerence=1e-8)
    with pytest.raises(TypeError, match="smoother_degre"):
        gmg.StokesMatrixFreeGPU(3, 2, {"smoother_degre": 6})  # raises before any CUDA call
    p = gmg.default_solve_params(linear_solver_tolerance=1e-8, restart=50, orthogonalization=1)
    assert (p.linear_solver_tolerance, p.restart, p.orthogonalization) == (1e-8, 50, 1)


def test_null_arrays_are_rejected_before_the_handle_is_used(L):
    """A null host array returns INVALID_ARGUMENT from the entry point's first
    line, before the handle is read (here a placeholder that is never one)."""
    fake = ctypes.create_string_buffer(64)
    h = ctypes.cast(fake, ctypes.c_void_p)
    x = np.zeros(8)
    p = x.ctypes.data_as(ctypes.c_void_p)
    out = gmg.Outputs()
    assert L.gb_gmg_vmult(h, 0, 0, 0, None, p) == INVALID
    assert L.gb_gmg_vmult(h, 0, 0, 0, p, None) == INVALID
    assert L.gb_gmg_vcycle(h, 0, 0, None, p) == INVALID
    assert L.gb_gmg_block_preconditioner(h, 0, p, None) == INVALID
    assert L.gb_gmg_transfer(h, 1, 0, 0, 1, None, p) == INVALID
    assert L.gb_gmg_solve(h, None, p, None, ctypes.byref(out)) == INVALID
    assert L.gb_gmg_solve(h, p, None, None, ctypes.byref(out)) == INVALID
    assert L.gb_gmg_adjoint_gradient(h, p, p, None) == INVALID
    assert L.gb_gmg_correct_stokes_rhs(h, None, p) == INVALID
    assert L.gb_gmg_assemble_rhs(h, p, None) == INVALID
    assert L.gb_gmg_solve_device(h, None, p, None, ctypes.byref(out)) == INVALID
    assert L.gb_gmg_solve_device(h, p, None, None, ctypes.byref(out)) == INVALID
    assert L.gb_gmg_vmult_device(h, 0, 0, None, p) == INVALID
    assert L.gb_gmg_vmult_device(h, 0, 0, p, None) == INVALID


def test_create_rejects_invalid_shapes(L):
    h = ctypes.c_void_p(1)
    for dim, deg, nl in [(1, 2, 3), (4, 2, 3), (3, 1, 3), (3, 4, 3), (3, 2, 0)]:
        assert L.gb_gmg_create(None, dim, deg, nl, ctypes.byref(h)) == INVALID
        assert h.value is None
    assert L.gb_gmg_create(None, 3, 2, 3, None) == INVALID


def test_null_handle_is_rejected_by_every_entry_point(L):
    x = np.zeros(8)
    p = x.ctypes.data_as(ctypes.c_void_p)
    prm = gmg.default_solve_params()
    out = gmg.Outputs()
    sec = ctypes.c_double()
    assert L.gb_gmg_vmult(None, 0, 0, 0, p, p) == INVALID
    assert L.gb_gmg_correct_stokes_rhs(None, p, p) == INVALID
    assert L.gb_gmg_solve(None, p, p, ctypes.byref(prm), ctypes.byref(out)) == INVALID
    assert L.gb_gmg_solve_device(None, p, p, ctypes.byref(prm), ctypes.byref(out)) == INVALID
    assert L.gb_gmg_adjoint_gradient(None, p, p, p) == INVALID
    assert L.gb_gmg_time_operation(None, 0, 0, 1, ctypes.byref(sec)) == INVALID
    assert L.gb_gmg_finalize_setup(None) == INVALID
    assert L.gb_gmg_build_preconditioner(None) == INVALID
    assert L.gb_gmg_set_viscosity(None, p, 1, 0, 1.0, 0) == INVALID
    assert L.gb_gmg_set_newton_terms(None, None) == INVALID
    assert L.gb_gmg_set_free_surface(None, 0, None, None, None, None) == INVALID
    assert L.gb_gmg_assemble_rhs(None, p, p) == INVALID
    L.gb_gmg_destroy(None)  # a no-op


def test_noalloc_entry_point_checks_before_touching_the_device(L):
    nc = (ctypes.c_int32 * 3)(4, 4, 4)
    h = (ctypes.c_double * 3)(0.25, 0.25, 0.25)
    dummy = ctypes.c_void_p(16)  # never dereferenced: every call below fails its checks first
    f = L.gb_gmg_ablock_apply_lattice_noalloc
    assert f(1, nc, h, 0, 1, dummy, dummy, dummy, None) == INVALID           # dim
    assert f(3, nc, h, 0, 5, dummy, dummy, dummy, None) == INVALID           # eta_per_cell not 1 or 27
    assert f(3, nc, h, 0, 1, None, dummy, dummy, None) == INVALID            # null viscosity
    bad = (ctypes.c_int32 * 3)(4, 0, 4)
    assert f(3, bad, h, 0, 1, dummy, dummy, dummy, None) == INVALID          # empty direction
    neg = (ctypes.c_double * 3)(0.25, -1.0, 0.25)
    assert f(3, nc, neg, 0, 1, dummy, dummy, dummy, None) == INVALID         # non-positive size
    big = (ctypes.c_int32 * 3)(17, 16, 16)                                   # 4352 > 4096 cells
    assert f(3, big, h, 0, 27, dummy, dummy, dummy, None) == EXCEEDS
    huge = (ctypes.c_int32 * 3)(2 ** 31 - 1, 2 ** 31 - 1, 2)                 # product beyond 64 bits
    assert f(3, huge, h, 0, 1, dummy, dummy, dummy, None) == EXCEEDS
    wrap = (ctypes.c_int32 * 3)(2 ** 16, 2 ** 16, 2 ** 16)                   # 2^48 cells
    assert f(3, wrap, h, 0, 1, dummy, dummy, dummy, None) == EXCEEDS


def test_no_gpu_means_no_solver():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gmg.GmgError) as e:
        gmg.StokesMatrixFreeGPU(3, 2)
    assert e.value.code == CUDA_ERROR


class _RecordingLibrary:
    """Stands in for the loaded library behind a front-end object: every entry
    point records its name and returns OK."""

    def __init__(self):
        self.calls = []

    def __getattr__(self, name):
        def entry(*args):
            self.calls.append(name)
            return OK
        return entry


def _front_end(degree=2):
    from types import SimpleNamespace

    g = object.__new__(gmg.StokesMatrixFreeGPU)  # no handle: nothing reaches a GPU
    g.L, g.h, g.dim, g.degree = _RecordingLibrary(), None, 3, degree
    g.levels = [SimpleNamespace(n_u=24, n_p=8, n_cells=1), SimpleNamespace(n_u=375, n_p=27, n_cells=8)]
    return g


def test_short_arrays_are_rejected_before_the_library_reads_them():
    """The library reads a fixed number of entries through each host pointer (the
    finest level's n_u + n_p for a solve, the operator's source size for a vmult,
    ...): the front end rejects a shorter array with INVALID_ARGUMENT before the
    call, and hands arrays of the used length (or longer) through."""
    g = _front_end()
    nu, npr, n = 375, 27, 402
    short = [
        lambda: g.solve(np.zeros(n - 1)),
        lambda: g.solve(np.zeros(n), x0=np.zeros(n - 1)),
        lambda: g.vmult(gmg.OP_STOKES, 1, np.zeros(n - 1)),
        lambda: g.vmult(gmg.OP_A, 0, np.zeros(23)),
        lambda: g.vmult(gmg.OP_BT, 1, np.zeros(npr - 1)),
        lambda: g.vcycle(0, np.zeros(nu - 1)),
        lambda: g.vcycle(1, np.zeros(npr - 1)),
        lambda: g.block_preconditioner(np.zeros(n - 1)),
        lambda: g.transfer(1, 0, True, np.zeros(nu - 1)),
        lambda: g.transfer(1, 1, False, np.zeros(7)),
        lambda: g.correct_stokes_rhs(np.zeros(n - 1), np.zeros(n)),
        lambda: g.adjoint_gradient(np.zeros(nu), np.zeros(nu - 1)),
        lambda: g.assemble_rhs(np.zeros((8, 27, 2))),
        lambda: g.set_eigenvalues(0, 0, gmg.FP64, [1.0]),
        lambda: g.assemble(np.ones(7), gmg.VISC_DGQ0, 1.0),
    ]
    for call in short:
        with pytest.raises(gmg.GmgError) as e:
            call()
        assert e.value.code == INVALID
    assert g.L.calls == []
    g.solve(np.zeros(n))
    g.vmult(gmg.OP_MASS, 1, np.zeros(npr))
    g.vcycle(0, np.zeros(nu))
    g.transfer(1, 0, False, np.zeros(24))
    g.adjoint_gradient(np.zeros(n), np.zeros(n))  # [u; p] vectors: the velocity part is read
    g.assemble_rhs(np.zeros((8, 27, 3)))
    assert g.L.calls == ["gb_gmg_solve", "gb_gmg_vmult", "gb_gmg_vcycle", "gb_gmg_transfer",
                         "gb_gmg_adjoint_gradient", "gb_gmg_assemble_rhs"]
    # degree 3: the body force is the library's to reject (it is built for degree 2)
    g3 = _front_end(degree=3)
    g3.assemble_rhs(np.zeros((8, 16, 3)))
    assert g3.L.calls == ["gb_gmg_assemble_rhs"]
