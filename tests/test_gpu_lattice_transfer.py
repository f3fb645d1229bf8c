"""Matrix-free level transfers between structured (lattice) levels: enabled on
every level pair of a lattice hierarchy (the set-up checks that the CSR
transfer matrices hold exactly the lattice stencils and reports it with
options.verbose), and equal to the CSR transfers of the same hierarchy with the
indexed layout (force_indexed_layout, CSR rows in another numbering, so equal
to rounding: FP64 1e-14, FP32 1e-6) for both blocks, both directions, 2D with
free-slip faces (SolCx) and 3D with no-slip faces (sinkers); the V-cycles of
the two handles agree as the lattice and indexed operators do."""
import numpy as np
import pytest

from aspect_gb300 import gmg, problems
from tests.gpu_util import rel_err

pytestmark = pytest.mark.gpu


def _problem(dim):
    return problems.solcx(5) if dim == 2 else problems.sinkers_3d(16, projection=1)


@pytest.mark.parametrize("dim", [2, 3])
def test_lattice_transfers_equal_csr(dim, capfd):
    P = _problem(dim)
    a = gmg.from_problem(P, {"verbose": 1})
    err = capfd.readouterr().err
    n_pairs = len(P.levels) - 1
    assert err.count("velocity lattice, pressure lattice") == n_pairs, err
    b = gmg.from_problem(P, {"force_indexed_layout": 1})
    rng = np.random.default_rng(3)
    for lev in range(1, len(P.levels)):
        c, f = P.levels[lev - 1], P.levels[lev]
        for block in (0, 1):
            xc = rng.normal(size=c.n_u if block == 0 else c.n_p)
            xf = rng.normal(size=f.n_u if block == 0 else f.n_p)
            for prec, tol in ((gmg.FP64, 1e-14), (gmg.FP32, 1e-6)):
                assert rel_err(a.transfer(lev, block, False, xc, prec), b.transfer(lev, block, False, xc, prec)) < tol
                assert rel_err(a.transfer(lev, block, True, xf, prec), b.transfer(lev, block, True, xf, prec)) < tol
    f = P.fine
    for block, n in ((0, f.n_u), (1, f.n_p)):
        r = rng.normal(size=n)
        assert rel_err(a.vcycle(block, r, gmg.FP64), b.vcycle(block, r, gmg.FP64)) < 1e-10
        assert rel_err(a.vcycle(block, r, gmg.FP32), b.vcycle(block, r, gmg.FP32)) < 1e-5
