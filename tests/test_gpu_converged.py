"""Convergence-driven stepping (main.cpp:1249-1271): sub-iterate until every
normalised change norm is below tol or max_subiters ran, then shift.

On the GPU the loop is a device-side while node of the step graph (or an
eager host loop); in a batch every case stops on its own test.  Checked
against the oracle's loop with the same test: equal sub-iteration counts,
bit-identical states."""
import numpy as np
import pytest

import oracle as O
from bcm_cgli_gb300 import api, cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def port():
    p = O.Port()
    p.set_threads(8)
    return p


def _same_state(a, y):
    for k, arr in zip(("U1_", "U1", "U1q"), y):
        x = getattr(a, k)
        bad = np.argwhere(x[1:] != arr[1:])
        assert bad.size == 0, f"{k}: {len(bad)} mismatches, first {bad[:3]}"


@pytest.mark.parametrize("graph", [False, True])
@pytest.mark.parametrize("method", [api.METHOD_RK3, api.METHOD_LUSGS])
def test_converged_single_case(port, graph, method):
    case = cases.random_two_level_case(seed=6, n=8, periodic=False)
    a = O.State(case)
    its_ref = port.run_converged(case, a, 3, 6 if method == api.METHOD_RK3 else 30, 0.02, method)
    ctx = api.CaseContext(case)
    ctx.set_method(method)
    ctx.set_state(case.U, case.U, case.U)
    er, its = ctx.advance_converged(3, 6 if method == api.METHOD_RK3 else 30, 0.02,
                                    use_graph=graph)
    assert list(its) == list(its_ref)
    _same_state(a, ctx.get_state())
    assert np.allclose(er[1:6], a.er[1:6], rtol=1e-12, atol=0)
    ctx.close()


@pytest.mark.parametrize("graph", [False, True])
def test_converged_batch_each_case_stops_on_its_own(port, graph):
    cs = [cases.taylor_green(ncx=2, n=8), cases.random_case(seed=3, n=8, periodic=True),
          cases.random_two_level_case(seed=6, n=8, periodic=False)]
    b = api.BatchContext(cs)
    b.set_method(api.METHOD_LUSGS)
    for q, c in enumerate(cs):
        b.set_case_state(q, c.U, c.U, c.U)
    er, its = b.advance_converged(2, 40, 0.02, use_graph=graph)
    assert its.shape == (2, 3)
    for q, c in enumerate(cs):
        a = O.State(c)
        ref = port.run_converged(c, a, 2, 40, 0.02, 1)
        assert list(its[:, q]) == list(ref), (c.name, its[:, q], ref)
        _same_state(a, b.get_case_state(q))
        assert np.allclose(er[q, 1:6], a.er[1:6], rtol=1e-12, atol=0)
    # the cases really stopped at different counts
    assert len(set(its[0])) > 1
    b.close()


def test_converged_split_batch_equals_solo():
    cs = [cases.taylor_green(ncx=2, n=8), cases.random_two_level_case(seed=6, n=8, periodic=False)]
    b = api.BatchContext(cs, precision=api.PRECISION_SPLIT)
    b.set_method(api.METHOD_LUSGS)
    for q, c in enumerate(cs):
        b.set_case_state(q, c.U, c.U, c.U)
    eb, ib = b.advance_converged(2, 40, 0.02)
    for q, c in enumerate(cs):
        s = api.CaseContext(c, precision=api.PRECISION_SPLIT)
        s.set_method(api.METHOD_LUSGS)
        s.set_state(c.U, c.U, c.U)
        es, is_ = s.advance_converged(2, 40, 0.02)
        assert list(is_) == list(ib[:, q])
        for x, y in zip(s.get_state(), b.get_case_state(q)):
            assert np.array_equal(x[1:], y[1:])
        assert np.array_equal(es[1:], eb[q, 1:])
        s.close()
    b.close()
