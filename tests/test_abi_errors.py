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
