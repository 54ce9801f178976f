"""LU-SGS (no reference counterpart): the CPU definition in the oracle
converges to the state the reference's RK sub-iterations converge to.

Both iterations solve R(Q) = 0 for the same discrete residual (BDF2 source,
inviscid and viscous fluxes) within a physical step, so run long enough they
must agree to round-off; LU-SGS gets there in far fewer sub-iterations."""
import numpy as np
import pytest

import oracle as O
from bcm_cgli_gb300 import cases


@pytest.fixture(scope="module")
def port():
    p = O.Port()
    p.set_threads(8)
    return p


def _interior(case, U):
    n = case.n
    fl = case.fws[1:, 2:n + 2, 2:n + 2, 2:n + 2] == 1
    return U[1:, 2:n + 2, 2:n + 2, 2:n + 2][fl]


def _rk_converged(port, case, subiters, ratio):
    st = O.State(case)
    old = case.dTau
    case.dTau = case.dT / ratio  # a larger pseudo-time step than the reference's dT/200
    try:
        port.run(case, st, 1, subiters)
    finally:
        case.dTau = old
    return st


def _rel(case, x, ref, U0):
    """Per-variable L2 distance relative to the step's change (momentum
    components relative to the momentum change's magnitude)."""
    sc = np.linalg.norm(ref - U0, axis=0)
    sc[1:4] = sc[1:4].max()
    return np.linalg.norm(x - ref, axis=0) / np.maximum(sc, 1e-300)


def test_lusgs_converges_to_the_rk_state_tgv(port):
    case = cases.taylor_green(ncx=2, n=8)
    ref = _interior(case, _rk_converged(port, case, 200, 2.0).U1)
    U0 = _interior(case, case.U)
    st = O.State(case)
    port.run_lusgs(case, st, 1, 16, 0.0, 1.0)
    assert _rel(case, _interior(case, st.U1), ref, U0).max() < 1e-9
    # the change norm of the last LU-SGS update is at round-off level
    assert st.er[1] < 1e-9


def test_lusgs_converges_to_the_rk_state_random_flags(port):
    """Random solid / IBM ghost flags, noise and IBM tables (omega 1.5)."""
    case = cases.random_case(seed=3, ncx=2, ncy=2, ncz=2, n=8, periodic=True)
    ref = _interior(case, _rk_converged(port, case, 300, 2.0).U1)
    U0 = _interior(case, case.U)
    errs = []
    for K in (16, 64):
        st = O.State(case)
        port.run_lusgs(case, st, 1, K, 0.0, 1.5)
        errs.append(_rel(case, _interior(case, st.U1), ref, U0).max())
    assert errs[1] < 1e-7 and errs[1] < errs[0] / 100


def test_lusgs_beats_rk_per_subiteration(port):
    """Same sub-iteration count: LU-SGS ends much closer to the converged
    state than RK at its stable pseudo-time step."""
    case = cases.random_case(seed=3, ncx=2, ncy=2, ncz=2, n=8, periodic=True)
    ref = _interior(case, _rk_converged(port, case, 300, 2.0).U1)
    U0 = _interior(case, case.U)
    rk = _interior(case, _rk_converged(port, case, 32, 2.0).U1)
    st = O.State(case)
    port.run_lusgs(case, st, 1, 32, 0.0, 1.5)
    lu = _interior(case, st.U1)
    assert _rel(case, lu, ref, U0).max() < _rel(case, rk, ref, U0).max() / 10
