"""The IBM ghost fill beside the boundary fill (bcmg_case_set_concurrent_ghosts).

For every case in which no IBM entry's cell (ghost cell or stencil) lies in
the three layers the boundary fill touches at a boundary face, a stage runs
that case's ghost-fill levels on a second stream while the boundary fill
runs, and the interface call waits for both.  The states must be the same bits as
with the fills one after the other, for FP64 and split precision, RK and
LU-SGS, eager launches, captured step graphs and convergence-driven graphs,
single cases and batches.
"""
import numpy as np
import pytest

from bcm_cgli_gb300 import api, cases
from golden import golden_cases as G

pytestmark = pytest.mark.gpu


def _sphere():
    return cases.sphere_ibm(n=8, coarse=2.0, box=((-2, 4), (-2, 2), (-2, 2)),
                            refine_box=((-2, 2), (-2, 2), (-2, 2)))


def _run(make_ctx, on, method, precision):
    ctx = make_ctx(precision)
    ctx.set_concurrent_ghosts(on)
    assert ctx.concurrent_ghosts() == on
    if method == "lusgs":
        ctx.set_method(api.METHOD_LUSGS)
    ctx.advance(1, 2, use_graph=False)
    ctx.advance(2, 2, use_graph=True)
    ctx.advance_converged(1, 4, tol=0.5)
    U = ctx.get_state()
    ctx.close()
    return U


def _single(precision):
    case = _sphere()
    ctx = api.CaseContext(case, precision=precision)
    ctx.set_state(case.U, case.U, case.U)
    return ctx


def _batch(precision):
    cs = [_sphere(), cases.sphere_ibm(n=8, coarse=2.0, box=((-2, 6), (-2, 2), (-4, 2)),
                                      refine_box=((-2, 2), (-2, 2), (-2, 2)), mach=0.4)]
    bt = api.BatchContext(cs, precision=precision)
    for q, c in enumerate(cs):
        bt.set_case_state(q, c.U, c.U, c.U)
    return bt


def _mixed(precision):
    """A sphere (beside) and a random case whose IBM cells sit next to
    boundary faces (in order), in one batch."""
    cs = [_sphere(), cases.random_case(seed=11, n=8, periodic=False, viscous=True)]
    bt = api.BatchContext(cs, precision=precision)
    for q, c in enumerate(cs):
        bt.set_case_state(q, c.U, c.U, c.U)
    return bt


@pytest.mark.parametrize("make", [_single, _batch, _mixed], ids=["sphere", "batch", "mixed"])
@pytest.mark.parametrize("method", ["rk3", "lusgs"])
@pytest.mark.parametrize("precision", [api.PRECISION_FP64, api.PRECISION_SPLIT])
def test_ghost_fill_beside_boundary_fill_changes_no_bit(make, method, precision):
    a = _run(make, True, method, precision)
    b = _run(make, False, method, precision)
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint64), y.view(np.uint64))


def test_not_beside_where_cells_are_shared():
    """The random test tables put IBM cells next to boundary faces: the fills
    stay in the reference's order there."""
    case = G.golden_cases()["random_open_n4"]
    ctx = api.CaseContext(case)
    assert not ctx.concurrent_ghosts()
    ctx.close()
