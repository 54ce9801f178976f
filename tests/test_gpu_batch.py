"""Batched cases: several independent cases (same n, different constants,
cube counts, time steps, boundaries, levels and IBM tables) advanced in one
context over a flat cube list.

FP64: every case's state is bit-identical to the oracle run of that case
alone, and its norms agree within 1e-12.  Split precision: every case's state
and norms are bit-identical to a split-precision context of that case alone
(the same per-cell arithmetic, the same per-case partial-sum order)."""
import numpy as np
import pytest

import oracle as O
from bcm_cgli_gb300 import api, cases

pytestmark = pytest.mark.gpu

NORM_RTOL = 1e-12
STEPS, SUBITERS = 2, 2


@pytest.fixture(scope="module")
def port():
    p = O.Port()
    p.set_threads(8)
    return p


def _mixed():
    """Four cases of n = 8 that differ in everything a batch may vary."""
    a = cases.random_case(seed=3, ncx=2, ncy=2, ncz=2, n=8, periodic=True, name="rand_periodic")
    b = cases.random_case(seed=4, ncx=3, ncy=2, ncz=1, n=8, periodic=False, name="rand_open")
    b.phys.rho0, b.phys.P0, b.phys.U0, b.phys.Uin = 1.05, 95000.0, 55.0, 52.0
    b.dT, b.dTau = 3e-4, 3e-4 / 150
    c = cases.sphere_cubes(64, n=8, mach=0.2, reynolds=150.0, seed=11)
    d = cases.isentropic_vortex(ncx=2, n=8)  # inviscid (mu_L = 0) inside a viscous batch
    e = cases.random_two_level_case(seed=9, n=8, periodic=False, name="two_level_open")
    e.phys.mpi_ncube = 5
    return [a, b, c, d, e]


def _norms_close(a, b, scale67):
    for m in range(1, 6):
        assert abs(a[m] - b[m]) <= NORM_RTOL * max(abs(b[m]), 1e-300), (m, a[m], b[m])
    for m in (6, 7):
        assert abs(a[m] - b[m]) <= NORM_RTOL * max(abs(b[m]), scale67), (m, a[m], b[m])


@pytest.mark.parametrize("graph", [False, True])
def test_fp64_batch_matches_each_case_alone(port, graph):
    cs = _mixed()
    ctx = api.BatchContext(cs)
    for q, c in enumerate(cs):
        ctx.set_case_state(q, c.U, c.U, c.U)
    er = ctx.advance(STEPS, SUBITERS, use_graph=graph)
    assert er.shape == (len(cs), 8)
    for q, c in enumerate(cs):
        a = O.State(c)
        port.run(c, a, STEPS, SUBITERS)
        U1_, U1, U1q = ctx.get_case_state(q)
        for k, y in (("U1_", U1_), ("U1", U1), ("U1q", U1q)):
            x = getattr(a, k)[1:]
            bad = np.argwhere(x != y[1:])
            assert bad.size == 0, f"{c.name} {k}: {len(bad)} mismatches, first {bad[:3]}"
        assert np.allclose(er[q, 1:6], a.er[1:6], rtol=NORM_RTOL, atol=0), (c.name, er[q], a.er)
        assert np.allclose(ctx.emax[q, 1:6], a.Emax[1:6], rtol=NORM_RTOL, atol=0)
        ph = c.phys
        scale = np.abs(a.Residual1).max() / (0.5 * ph.rho0 * ph.U0 ** 2 * 2.602)
        assert abs(er[q, 6] - a.er[6]) <= NORM_RTOL * max(abs(a.er[6]), scale)
        assert abs(er[q, 7] - a.er[7]) <= NORM_RTOL * max(abs(a.er[7]), scale)
    ctx.close()


def test_split_batch_equals_split_single_contexts():
    cs = _mixed()
    bctx = api.BatchContext(cs, precision=api.PRECISION_SPLIT)
    for q, c in enumerate(cs):
        bctx.set_case_state(q, c.U, c.U, c.U)
    er = bctx.advance(STEPS, SUBITERS)
    for q, c in enumerate(cs):
        sctx = api.CaseContext(c, precision=api.PRECISION_SPLIT)
        sctx.set_state(c.U, c.U, c.U)
        es = sctx.advance(STEPS, SUBITERS)
        ys = sctx.get_state()
        yb = bctx.get_case_state(q)
        for k in range(3):
            assert np.array_equal(ys[k][1:], yb[k][1:]), (c.name, k)
        assert np.array_equal(es[1:], er[q, 1:]), (c.name, es, er[q])
        sctx.close()
    bctx.close()


def test_batch_of_one_equals_single_context():
    c = cases.random_two_level_case(seed=2, n=8, periodic=True)
    s = api.CaseContext(c)
    s.set_state(c.U, c.U, c.U)
    es = s.advance(1, 3)
    b = api.BatchContext([c])
    b.set_case_state(0, c.U, c.U, c.U)
    eb = b.advance(1, 3)
    for x, y in zip(s.get_state(), b.get_case_state(0)):
        assert np.array_equal(x[1:], y[1:])
    assert np.allclose(eb[0, 1:6], es[1:6], rtol=NORM_RTOL, atol=0)
    assert b.case_cubes(0) == (1, c.ncube)
    s.close()
    b.close()


def test_batch_cube_numbering_and_whole_state():
    cs = _mixed()[:3]
    b = api.BatchContext(cs)
    g = 1
    for q, c in enumerate(cs):
        assert b.case_cubes(q) == (g, c.ncube)
        g += c.ncube - 1
    assert b.shape[0] == g
    for q, c in enumerate(cs):
        b.set_case_state(q, c.U, c.U, c.U)
    U1_, _, _ = b.get_state()
    for q, c in enumerate(cs):
        g0, nq = b.case_cubes(q)
        assert np.array_equal(U1_[g0:g0 + nq - 1], c.U[1:])
    b.close()
