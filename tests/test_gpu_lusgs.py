"""LU-SGS on the GPU (no reference counterpart).

The kernel sweeps each cube's planes i+j+k = const in parallel; every cell's
arithmetic equals the oracle's serial lexicographic sweep, so the state after
whole dual-time steps is bit-identical to the oracle's LU-SGS run (norms
within 1e-12, their sum order differs).  Converged, it equals the RK
sub-iterations' state."""
import numpy as np
import pytest

import oracle as O
from bcm_cgli_gb300 import api, cases
from golden import golden_cases as G

pytestmark = pytest.mark.gpu

NAMES = sorted(G.golden_cases())


@pytest.fixture(scope="module")
def port():
    p = O.Port()
    p.set_threads(8)
    return p


def _check(case, a, ctx_state, er, emax):
    U1_, U1, U1q = ctx_state
    for k, y in (("U1_", U1_), ("U1", U1), ("U1q", U1q)):
        x = getattr(a, k)
        bad = np.argwhere(x[1:] != y[1:])
        assert bad.size == 0, f"{case.name} {k}: {len(bad)} mismatches, first {bad[:3]}"
    assert np.allclose(er[1:6], a.er[1:6], rtol=1e-12, atol=0), (er, a.er)
    assert np.allclose(emax[1:6], a.Emax[1:6], rtol=1e-12, atol=0)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("graph", [False, True])
def test_lusgs_bitwise_against_oracle(port, name, graph):
    case = G.golden_cases()[name]
    a = O.State(case)
    port.run_lusgs(case, a, 2, 3, 0.0, 1.5)
    ctx = api.CaseContext(case)
    ctx.set_method(api.METHOD_LUSGS, cfl=0.0, omega=1.5)
    ctx.set_state(case.U, case.U, case.U)
    er = ctx.advance(2, 3, use_graph=graph)
    _check(case, a, ctx.get_state(), er, ctx.emax)
    assert ctx.launch_count() > 0
    ctx.close()


def test_lusgs_bitwise_sphere_with_pseudo_time(port):
    """Two-level sphere with IBM ghost cells, open boundaries and a finite
    pseudo-time CFL."""
    case = cases.sphere_cubes(64, n=8, mach=0.2, reynolds=150.0, seed=11)
    a = O.State(case)
    port.run_lusgs(case, a, 1, 3, 5.0, 2.0)
    ctx = api.CaseContext(case)
    ctx.set_method(api.METHOD_LUSGS, cfl=5.0, omega=2.0)
    ctx.set_state(case.U, case.U, case.U)
    er = ctx.advance(1, 3)
    _check(case, a, ctx.get_state(), er, ctx.emax)
    ctx.close()


def test_lusgs_batch_bitwise_per_case(port):
    cs = [cases.random_case(seed=5, n=8, periodic=True, name="a"),
          cases.random_two_level_case(seed=6, n=8, periodic=False, name="b"),
          cases.taylor_green(ncx=2, n=8)]
    cs[1].dT = 3e-4
    b = api.BatchContext(cs)
    b.set_method(api.METHOD_LUSGS)
    for q, c in enumerate(cs):
        b.set_case_state(q, c.U, c.U, c.U)
    er = b.advance(1, 4)
    for q, c in enumerate(cs):
        a = O.State(c)
        port.run_lusgs(c, a, 1, 4, 0.0, 1.5)
        _check(c, a, b.get_case_state(q), er[q], b.emax[q])
    b.close()


def test_lusgs_converges_to_rk_state_on_gpu():
    case = cases.taylor_green(ncx=2, n=8)
    n = case.n
    rk = api.CaseContext(case)
    old = case.dTau
    case.dTau = case.dT / 2.0
    rk2 = api.CaseContext(case)  # RK with a larger pseudo-time step
    case.dTau = old
    rk.close()
    rk2.set_state(case.U, case.U, case.U)
    rk2.advance(1, 200)
    ref = rk2.get_state()[1][1:, 2:n + 2, 2:n + 2, 2:n + 2].reshape(-1, 5)
    lu = api.CaseContext(case)
    lu.set_method(api.METHOD_LUSGS, omega=1.0)
    lu.set_state(case.U, case.U, case.U)
    lu.advance(1, 16)
    x = lu.get_state()[1][1:, 2:n + 2, 2:n + 2, 2:n + 2].reshape(-1, 5)
    U0 = case.U[1:, 2:n + 2, 2:n + 2, 2:n + 2].reshape(-1, 5)
    sc = np.linalg.norm(ref - U0, axis=0)
    sc[1:4] = sc[1:4].max()
    assert (np.linalg.norm(x - ref, axis=0) / sc).max() < 1e-9
    rk2.close()
    lu.close()


def test_lusgs_rejects_bad_settings():
    case = cases.random_case(seed=1, n=4, periodic=True)
    ctx = api.CaseContext(case)
    with pytest.raises(api.BcmgError):
        ctx.set_method(api.METHOD_LUSGS, omega=0.5)
    with pytest.raises(api.BcmgError):
        ctx.set_method(7)
    ctx.close()


def _rel_l2_scaled(a, b, n):
    ai = a[1:, 2:n + 2, 2:n + 2, 2:n + 2].reshape(-1, 5)
    bi = b[1:, 2:n + 2, 2:n + 2, 2:n + 2].reshape(-1, 5)
    d = np.linalg.norm(ai - bi, axis=0)
    own = d / np.maximum(np.linalg.norm(bi, axis=0), 1e-300)
    mom = np.linalg.norm(bi[:, 1:4])
    return np.array([own[0], d[1] / mom, d[2] / mom, d[3] / mom, own[4]])


@pytest.mark.parametrize("make", [lambda: cases.taylor_green(ncx=2, n=8),
                                  lambda: cases.sphere_cubes(64, n=8, mach=0.2, reynolds=150.0,
                                                             seed=11)])
def test_split_lusgs_close_to_fp64_lusgs(make):
    """FP32 sweeps on the FP32 mirror: after a dual-time step of LU-SGS
    sub-iterations the state is within the split path's 1e-5 bound of the
    FP64 LU-SGS state (relative L2, momentum scaled by its magnitude)."""
    case = make()
    out = {}
    for prec in (api.PRECISION_FP64, api.PRECISION_SPLIT):
        ctx = api.CaseContext(case, precision=prec)
        ctx.set_method(api.METHOD_LUSGS)
        ctx.set_state(case.U, case.U, case.U)
        out[prec] = (ctx.advance(2, 8), ctx.get_state()[0])
        ctx.close()
    err = _rel_l2_scaled(out[api.PRECISION_SPLIT][1], out[api.PRECISION_FP64][1], case.n)
    assert err.max() < 1e-5, err


def test_split_lusgs_batch_equals_single():
    cs = [cases.taylor_green(ncx=2, n=8), cases.random_two_level_case(seed=6, n=8, periodic=False)]
    b = api.BatchContext(cs, precision=api.PRECISION_SPLIT)
    b.set_method(api.METHOD_LUSGS, omega=1.5)
    for q, c in enumerate(cs):
        b.set_case_state(q, c.U, c.U, c.U)
    eb = b.advance(1, 4)
    for q, c in enumerate(cs):
        s = api.CaseContext(c, precision=api.PRECISION_SPLIT)
        s.set_method(api.METHOD_LUSGS, omega=1.5)
        s.set_state(c.U, c.U, c.U)
        es = s.advance(1, 4)
        for x, y in zip(s.get_state(), b.get_case_state(q)):
            assert np.array_equal(x[1:], y[1:])
        assert np.array_equal(es[1:], eb[q, 1:])
        s.close()
    b.close()
