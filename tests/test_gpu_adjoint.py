"""Adjoint viscosity gradient on the GPU (FP32 V-cycle, FP64 outer solves):
central finite differences (eps 1e-6, 20 seeded directions, 1e-5 relative) on
the 32^3 workload and on 8^3, the FP64 CPU adjoint (oracle solves and oracle
gradient), and the torch.autograd shim."""
import numpy as np
import pytest

from aspect_gb300 import adjoint, gmg
from oracle import Oracle
from tests.test_adjoint_cpu import OracleEvaluator

pytestmark = pytest.mark.gpu


def _factory(base):
    g = gmg.StokesMatrixFreeGPU(3, len(base.levels))
    g.setup_dofs(base.levels)
    return g


@pytest.fixture(scope="module", params=[8, 32])
def problem(request):
    return adjoint.make_problem(request.param, _factory)


def test_gradient_matches_central_differences(problem):
    """The gradient comes from FP32-V-cycle / FP64-outer forward and adjoint
    solves; the finite-difference reference evaluates J with FP64 V-cycles to a
    1e-13 relative residual (an eps = 1e-6 difference quotient needs J to about
    1e-13), both solves of a pair sharing the preconditioner built at ln(eta)."""
    ap, ev = problem
    J, g, _, _ = ev.gradient(ap.lneta)
    assert J > 0
    fd_ev = adjoint.Evaluator(ev.g, ap.base, ap.u_obs, ap.top, tol=1e-13, mg_precision=gmg.FP64)
    fd_ev.forward(ap.lneta)  # builds the shared preconditioner
    eps = 1e-6
    dirs = adjoint.fd_directions(len(ap.lneta), 20, adjoint.SEED_A + 100)
    fd = np.array([(fd_ev.forward(ap.lneta + eps * d, keep_preconditioner=True)[1]
                    - fd_ev.forward(ap.lneta - eps * d, keep_preconditioner=True)[1]) / (2 * eps) for d in dirs])
    gd = dirs @ g
    # relative error over the 20 directions (a single direction nearly orthogonal
    # to g would make a per-direction ratio meaningless), and per direction
    # against the scale |g| |d| of a directional derivative
    assert np.linalg.norm(fd - gd) <= 1e-5 * np.linalg.norm(gd), (fd, gd)
    assert np.all(np.abs(fd - gd) <= 1e-5 * np.linalg.norm(g)), np.abs(fd - gd) / np.linalg.norm(g)


def test_gradient_matches_fp64_cpu_adjoint():
    ap, ev = adjoint.make_problem(8, _factory)
    J, g, _, _ = ev.gradient(ap.lneta)
    cpu = OracleEvaluator(ap.base, ap.top, ap.u_obs)
    Jc, gc = cpu.gradient(ap.lneta)
    assert abs(J - Jc) <= 1e-9 * abs(Jc)
    assert np.linalg.norm(g - gc) <= 1e-7 * np.linalg.norm(gc)


def test_torch_autograd_shim():
    torch = pytest.importorskip("torch")
    ap, ev = adjoint.make_problem(8, _factory)
    fn = adjoint.torch_misfit_function()
    x = torch.tensor(ap.lneta, dtype=torch.float64, requires_grad=True)
    J = fn.apply(x, ev)
    J.backward()
    _, g, _, _ = ev.gradient(ap.lneta)
    assert torch.allclose(x.grad, torch.as_tensor(g), rtol=1e-10, atol=0)
