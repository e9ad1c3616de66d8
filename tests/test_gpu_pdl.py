"""Programmatic dependent launch (gb_set_pdl) changes only how the solver-loop kernels are scheduled:
the multigrid V-cycle, the graph-captured learned flexible-CG solve and the refined Jacobi-CG solve
give bit-identical results with it on and off."""

import os

import pytest
import torch

pytestmark = pytest.mark.gpu

WEIGHTS = os.path.join(os.path.dirname(__file__), "..", "warp_gb300", "data", "smoother_q1_diffusion.npz")


@pytest.fixture
def pdl_switch():
    from warp_gb300 import _native as N

    before = N.lib().gb_get_pdl()
    yield lambda mode: N.call("gb_set_pdl", int(mode))
    N.call("gb_set_pdl", before)


def test_pdl_is_on_by_default_and_switchable(cuda, pdl_switch):
    from warp_gb300 import _native as N

    assert N.lib().gb_get_pdl() in (0, 1, 2)
    pdl_switch(0)
    assert N.lib().gb_get_pdl() == 0
    pdl_switch(2)
    assert N.lib().gb_get_pdl() == 2
    pdl_switch(1)
    assert N.lib().gb_get_pdl() == 1
    assert N.lib().gb_set_pdl(3) != 0  # out of range


def _solve(system, method, graph, pdl_switch, on):
    from warp_gb300 import learned, multigrid
    from warp_gb300.optim import linear

    pdl_switch(on)
    if method == "jacobi":
        solver = linear.RefinedSolver(system.A, M=linear.preconditioner(system.A, "diag"), inner_tol=1e-5,
                                      use_cuda_graph=graph)
        mg = None
    else:
        mg = multigrid.MultigridPreconditioner(system.A, system.geo, system.coef)
        if method == "learned":
            mg.smoother = learned.LearnedSmoother(learned.ConvNet.load(WEIGHTS), mg, system.coef, backend="tc")
        solver = linear.RefinedSolver(system.A, M=mg, method="fcg", inner_tol=1e-5, use_cuda_graph=graph)
    r = torch.randn(system.A.nrow, device="cuda", generator=torch.Generator("cuda").manual_seed(5))
    z = mg.apply(r * (1 - mg.levels[0].mask)) if mg is not None else None
    x, info = solver.solve(system.b, tol=1e-8)
    torch.cuda.synchronize()
    if mg is not None:
        assert int(mg.status.item()) == 0
    return x, info, z


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("method", ["jacobi", "mg", "learned"])
def test_pdl_results_are_bit_identical(cuda, pdl_switch, method, graph, mode):
    """Mode 1: eager launches (graph=False) run with the programmatic-serialization attribute, graph
    captures stay plain; mode 2: captures carry it too.  No mode may change a bit."""
    from warp_gb300 import problems

    system = problems.diffusion((24, 24, 24), sigma=1.5, corr_length=0.15, seed=4)
    x_off, info_off, z_off = _solve(system, method, graph, pdl_switch, 0)
    x_on, info_on, z_on = _solve(system, method, graph, pdl_switch, mode)
    assert info_on["converged"] and info_off["converged"]
    assert info_on["inner_iterations"] == info_off["inner_iterations"]
    assert torch.equal(x_on, x_off)
    if z_on is not None:
        assert torch.equal(z_on, z_off)
