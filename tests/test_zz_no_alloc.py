"""The allocation-free A-block entry point against the handle-based one.

gb_gmg_ablock_apply_lattice_noalloc serves callers that cannot call cudaMalloc
when they need the operator (code under a device-memory budget owned by another
allocator, code that must not block on the driver's allocator); its per-cell
scratch is a static device array shared by all calls. Checked here through the C ABI against
gb_gmg_vmult (FP32 A block) on the same lattice levels, on two calls in a row so
that a call cannot lean on what the previous one left in the shared array.
This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

from aspect_gb300 import gmg, mesh

pytestmark = pytest.mark.gpu

TOL32 = 2e-6


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _zero_faces(dim):
    """Free slip on every face: the normal component is zero."""
    bits = 0
    for c in range(dim):
        for side in (0, 1):
            bits |= 1 << ((2 * c + side) * 3 + c)
    return bits


def _noalloc(torch, dim, n, eta, x):
    d_eta = torch.from_numpy(np.ascontiguousarray(eta, dtype=np.float32).ravel()).cuda()
    d_src = torch.from_numpy(x.astype(np.float32)).cuda()
    d_dst = torch.full_like(d_src, float("nan"))
    ncd = np.full(dim, n, dtype=np.int32)
    h = np.full(dim, 1.0 / n)
    stream = torch.cuda.current_stream().cuda_stream
    rc = gmg.load_library().gb_gmg_ablock_apply_lattice_noalloc(
        dim, ctypes.c_void_p(ncd.ctypes.data), ctypes.c_void_p(h.ctypes.data), _zero_faces(dim),
        eta.shape[1] if eta.ndim == 2 else 1, ctypes.c_void_p(d_eta.data_ptr()), ctypes.c_void_p(d_src.data_ptr()),
        ctypes.c_void_p(d_dst.data_ptr()), ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, d_dst.double().cpu().numpy()


@pytest.mark.parametrize("dim,n,per_q", [(3, 8, True), (3, 16, False), (2, 32, True)])
def test_noalloc_matches_handle_entry_point(dim, n, per_q):
    torch = pytest.importorskip("torch")
    levels = mesh.box_hierarchy(dim, n)
    fine = levels[-1]
    rng = np.random.default_rng(dim * 100 + n)
    nq = 3 ** dim
    eta = np.exp(3 * rng.uniform(-1, 1, size=(fine.n_cells, nq) if per_q else fine.n_cells))
    g = gmg.StokesMatrixFreeGPU(dim, len(levels))
    g.setup_dofs(levels)
    g.assemble(eta, gmg.VISC_DGQ0, 1.0)
    top = len(levels) - 1
    for call in range(2):
        x = rng.normal(size=fine.n_u).astype(np.float32).astype(np.float64)
        y_ref = g.vmult(gmg.OP_A, top, x, gmg.FP32)
        rc, y = _noalloc(torch, dim, n, eta if per_q else eta[:, None], x)
        assert rc == 0, (call, rc)
        assert _rel(y, y_ref) < TOL32, (call, _rel(y, y_ref))


def test_noalloc_rejects_levels_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    n = 17  # 4913 cells > GB_GMG_NOALLOC_MAX_CELLS
    n_u = 3 * (2 * n + 1) ** 3
    rc, y = _noalloc(torch, 3, n, np.ones((n ** 3, 1)), np.ones(n_u))
    assert rc == 8  # GB_GMG_EXCEEDS_STATIC_SCRATCH
    assert np.isnan(y).all()  # nothing was written
