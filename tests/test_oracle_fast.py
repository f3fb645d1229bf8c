"""The oracle's fast mode (sum-factorised cell operators and parallel
reductions, used to time the CPU baseline) against its plain quadrature loops
(the checker): same operators to rounding, same diagonals, same solves."""
import numpy as np
import pytest

import oracle
from aspect_gb300 import problems
from oracle import Oracle
from tests.gpu_util import hierarchy, random_eta


@pytest.fixture
def fast_off():
    yield
    oracle.set_fast(False)


@pytest.mark.parametrize("dim,n,geometry,per_q,compressible", [
    (3, 4, "box", True, 0), (3, 4, "q2-distorted", False, 1), (2, 8, "box", True, 0),
    (2, 8, "q2-distorted", True, 1), (3, 4, "q2", True, 0)])
def test_fast_operators_match_plain(fast_off, dim, n, geometry, per_q, compressible):
    levels = hierarchy(dim, n, geometry=geometry, permute=True)
    o = Oracle(levels)
    o.set_viscosity(random_eta(levels[-1], per_q), 0, 1.7, compressible)
    f = levels[-1]
    top = len(levels) - 1
    x = np.random.default_rng(1).normal(size=f.n_u + f.n_p)
    for op, src in ((0, x), (1, x[: f.n_u]), (2, x[f.n_u:]), (3, x[f.n_u:])):
        oracle.set_fast(False)
        a = o.vmult(op, top, src)
        oracle.set_fast(True)
        b = o.vmult(op, top, src)
        assert np.linalg.norm(a - b) <= 1e-13 * np.linalg.norm(a), op


def test_fast_diagonals_and_solve_match_plain(fast_off):
    P = problems.sinkers_3d(8)
    res = {}
    for fast in (False, True):
        oracle.set_fast(fast)
        o = Oracle(P.levels)
        o.set_viscosity(P.eta, P.projection, P.pressure_scaling)
        o.build_preconditioner(False)
        d = [o.diagonal_inverse(len(P.levels) - 1, b) for b in (0, 1)]
        x, info = o.solve(P.rhs, tol_rel=1e-8)
        res[fast] = (d, x, info)
    (d0, x0, i0), (d1, x1, i1) = res[False], res[True]
    for a, b in zip(d0, d1):
        np.testing.assert_allclose(b, a, rtol=1e-13)
    assert i0["status"] == 0 and i1["status"] == 0
    assert i0["cheap_iterations"] == i1["cheap_iterations"]
    assert np.linalg.norm(x1 - x0) <= 1e-8 * np.linalg.norm(x0)
