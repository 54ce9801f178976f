"""GPU parity: the CUDA path (through the C ABI) against the oracle.

The FP64 path is bit-identical to the reference, so state arrays are
compared with exact equality (signed zeros compare equal).  The residual
norms are sums whose order differs from the reference's serial loop, so they
are compared with a relative tolerance of 1e-12 (the FP64 path's stated
tolerance)."""
import numpy as np
import pytest

import oracle as O
from bcm_cgli_gb300 import api, cases
from golden import golden_cases as G

pytestmark = pytest.mark.gpu

NORM_RTOL = 1e-12
NAMES = sorted(G.golden_cases())


@pytest.fixture(scope="module")
def port():
    p = O.Port()
    p.set_threads(8)
    return p


def _cases():
    return G.golden_cases()


def assert_norms_close(a, b, resid=None):
    a, b = np.asarray(a), np.asarray(b)
    for m in range(1, 6):
        assert abs(a[m] - b[m]) <= NORM_RTOL * max(abs(a[m]), 1e-300), (m, a[m], b[m])
    for m in (6, 7):
        # force sums: tolerance relative to the sum of magnitudes
        scale = max(abs(a[m]), 1e-300)
        if resid is not None:
            scale = max(scale, np.abs(resid).max())
        assert abs(a[m] - b[m]) <= NORM_RTOL * scale, (m, a[m], b[m])


@pytest.mark.parametrize("name", NAMES)
def test_flux_twin_bitwise(port, name):
    case = _cases()[name]
    api.reference_config_for(case)
    a, b = O.State(case), O.State(case)
    for RK in (1, 2, 3):
        port.flux_stage(case, a, RK)
        api.BCM_Flux_XYZ_Viscous_Runge_kutta(0, case.ncube, RK, case.dT, case.dTau, case.e,
                                             case.fws, case.csl, case.cube_size, b.U1_, b.U1,
                                             b.U1q, b.U1p1, b.U1p2, b.Rku1, b.Residual1, b.er)
        for k in ("U1_", "Rku1", "Residual1", "U1p1", "U1p2"):
            x, y = getattr(a, k), getattr(b, k)
            bad = np.argwhere(x != y)
            assert bad.size == 0, f"{name} RK{RK} {k}: {len(bad)} mismatches, first {bad[:3]}"
    assert_norms_close(a.er, b.er)


@pytest.mark.parametrize("name", NAMES)
def test_boundary_twins_bitwise(port, name):
    case = _cases()[name]
    api.reference_config_for(case)
    a, b = O.State(case), O.State(case)
    port.bc(case, a.U1_)
    xl, xu, yl, yu, zl, zu = (api._one_based(x) for x in case.bc_lists())
    api.BCM_X_boundary_condition(0, len(xl) - 1, len(xu) - 1, xl, xu, b.U1_)
    api.BCM_Y_boundary_condition(len(yl) - 1, len(yu) - 1, yl, yu, b.U1_)
    api.BCM_Z_boundary_condition(len(zl) - 1, len(zu) - 1, zl, zu, b.U1_)
    assert np.array_equal(a.U1_, b.U1_)


@pytest.mark.parametrize("name", NAMES)
def test_ghostcell_twins_bitwise(port, name):
    case = _cases()[name]
    if case.ibm_minus is None:
        pytest.skip("no IBM tables in this case")
    api.reference_config_for(case)
    a, b = O.State(case), O.State(case)
    port.ghost(case, a.U1_, -1)
    port.ghost(case, a.U1_, 1)
    for which, t in ((-1, case.ibm_minus), (1, case.ibm_plus)):
        W, Gi, I = t
        f = api.BCM_Ghostcell_minus if which < 0 else api.BCM_Ghostcell_plus
        f(0, (len(Gi) - 1) // 4, W, Gi, I, case.fws, b.U1_)
    assert np.array_equal(a.U1_, b.U1_)


@pytest.mark.parametrize("name", NAMES)
def test_interface_twin_bitwise(port, name):
    case = _cases()[name]
    api.reference_config_for(case)
    a, b = O.State(case), O.State(case)
    port.interface(case, a.U1_)
    api.BCM_Interface_for_case(case, b.U1_)
    assert np.array_equal(a.U1_, b.U1_)


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("graph", [False, True])
def test_resident_loop_bitwise(port, name, graph):
    case = _cases()[name]
    a = O.State(case)
    port.run(case, a, G.RUN_STEPS, G.RUN_SUBITERS)
    ctx = api.CaseContext(case)
    ctx.set_state(case.U, case.U, case.U)
    er = ctx.advance(G.RUN_STEPS, G.RUN_SUBITERS, use_graph=graph)
    U1_, U1, U1q = ctx.get_state()
    for k, y in (("U1_", U1_), ("U1", U1), ("U1q", U1q)):
        x = getattr(a, k)
        bad = np.argwhere(x != y)
        assert bad.size == 0, f"{name} {k}: {len(bad)} mismatches, first {bad[:3]}"
    # er[1..5] are normalised by their running maxima (main.cpp:1249-1259)
    assert np.allclose(er[1:6], a.er[1:6], rtol=1e-12, atol=0)
    assert np.allclose(ctx.emax[1:6], a.Emax[1:6], rtol=NORM_RTOL, atol=0)
    assert ctx.launch_count() > 0
    ctx.close()


def test_stage_scratch_bitwise(port):
    """Rku1 / Residual1 / U1p1 / U1p2 of the resident stage equal the oracle's."""
    case = _cases()["random_open_n4"]
    a = O.State(case)
    ctx = api.CaseContext(case)
    ctx.set_state(case.U, case.U, case.U)
    for RK in (1, 2, 3):
        port.bc(case, a.U1_)
        port.ghost(case, a.U1_, -1)
        port.ghost(case, a.U1_, 1)
        port.interface(case, a.U1_)
        port.flux_stage(case, a, RK)
        port.interface(case, a.U1_)
        ctx.stage(RK)
        U1p1, U1p2, Rku1, Res = ctx.get_scratch()
        U1_ = ctx.get_state()[0]
        for k, y in (("U1_", U1_), ("U1p1", U1p1), ("U1p2", U1p2), ("Rku1", Rku1),
                     ("Residual1", Res)):
            assert np.array_equal(getattr(a, k), y), (RK, k)
    ctx.close()


def test_full_size_tgv_sampled_cubes(port):
    """Config-2 size (8^3 cubes of 24^3 cells, 7.1M cells): one GPU flux stage
    over the whole case; a sample of cubes is recomputed by the oracle on its
    own from the same inputs and must match bit for bit (a cube's increment
    depends only on its own padded block)."""
    case = cases.taylor_green(ncx=8, n=24)
    api.reference_config_for(case)
    b = O.State(case)
    api.BCM_Interface_for_case(case, b.U1_)
    api.BCM_Flux_XYZ_Viscous_Runge_kutta(0, case.ncube, 1, case.dT, case.dTau, case.e, case.fws,
                                         case.csl, case.cube_size, b.U1_, b.U1, b.U1q, b.U1p1,
                                         b.U1p2, b.Rku1, b.Residual1, b.er)
    rng = np.random.default_rng(7)
    pick = np.sort(rng.choice(np.arange(1, case.ncube), size=6, replace=False))
    # A sub-case made of the picked cubes (slot 0 unused), fed the GPU's
    # post-interface input state of those cubes.
    sub = cases.Case(n=case.n, ncube=len(pick) + 1, phys=case.phys,
                     cube_size=np.concatenate([[0.0], case.cube_size[pick]]),
                     csl=np.concatenate([[0], case.csl[pick]]).astype(np.int32),
                     origin=np.zeros((len(pick) + 1, 3)),
                     adj=np.zeros((len(pick) + 1, 5, 7), np.int32),
                     fws=np.ascontiguousarray(np.concatenate([case.fws[:1], case.fws[pick]])),
                     U=np.zeros((len(pick) + 1,) + case.U.shape[1:]),
                     dT=case.dT, dTau=case.dTau, e=case.e)
    a = O.State(sub)
    pre = O.State(case)
    api.BCM_Interface_for_case(case, pre.U1_)
    a.U1_[1:] = pre.U1_[pick]
    a.U1[1:] = case.U[pick]
    a.U1q[1:] = case.U[pick]
    port.flux_stage(sub, a, 1)
    assert np.array_equal(a.Rku1[1:], b.Rku1[pick])
    assert np.array_equal(a.U1_[1:], b.U1_[pick])


@pytest.mark.parametrize("workload", ["tgv", "sphere"])
def test_full_size_loop_bitwise(port, workload):
    """Full benchmark sizes: config 2 (TGV, 8^3 cubes of 24^3, 7.1 M cells)
    and config 3 (1,584 cubes of 16^3 on two levels, 6.5 M cells, IBM tables
    from the GPU preprocessing of the 20,480-triangle body, open-domain
    boundaries): one FP64 dual-time step of two sub-iterations, replayed as one
    graph, equals the oracle's loop bit for bit in every state array."""
    if workload == "tgv":
        case = cases.taylor_green(ncx=8, n=24)
    else:
        case = cases.sphere_ibm(preprocess=api.ibm_preprocess)
    a = O.State(case)
    port.run(case, a, 1, 2)
    ctx = api.CaseContext(case)
    ctx.set_state(case.U, case.U, case.U)
    er = ctx.advance(1, 2, use_graph=True)
    U1_, U1, U1q = ctx.get_state()
    for k, y in (("U1_", U1_), ("U1", U1), ("U1q", U1q)):
        bad = np.argwhere(getattr(a, k) != y)
        assert bad.size == 0, f"{k}: {len(bad)} mismatches, first {bad[:3]}"
    # The norms are ratios of sums over ~7 M cells taken in different orders
    # (fixed GPU blocks against the oracle's thread chunks); the rounding bound
    # of such a sum is about n * 2^-53 = 7e-10 relative (observed: 1.3e-12).
    rel = np.max(np.abs(er[1:6] - a.er[1:6]) / np.abs(a.er[1:6]))
    assert rel <= 7e-10, rel
    ctx.close()


def test_invalid_inputs_fail_loudly():
    case = cases.random_case(seed=3, n=4)
    W, Gi, I = case.ibm_minus
    I = I.copy()
    I[2] = case.S  # stencil outside the padded cube
    case.ibm_minus = (W, Gi, I)
    with pytest.raises(api.BcmgError):
        api.CaseContext(case)
    bad = cases.random_case(seed=3, n=4)
    bad.adj = bad.adj.copy()
    bad.adj[1, 1, 2] = bad.ncube + 5
    with pytest.raises(api.BcmgError):
        api.CaseContext(bad)
    api.reference_config_for(cases.random_case(seed=3, n=4))
    U = cases.random_case(seed=3, n=4).U.copy()
    with pytest.raises(api.BcmgError):
        api.BCM_X_boundary_condition(0, 1, 0, np.array([0, 99], np.int32)[:1].repeat(2) * 0 - 1,
                                     np.zeros(1, np.int32), U)


def _small_sphere():
    return cases.sphere_ibm(n=8, coarse=2.0, box=((-2, 4), (-2, 2), (-2, 2)),
                            refine_box=((-2, 2), (-2, 2), (-2, 2)))


@pytest.mark.parametrize("precision", [api.PRECISION_FP64, api.PRECISION_SPLIT])
@pytest.mark.parametrize("method", [api.METHOD_RK3, api.METHOD_LUSGS])
@pytest.mark.parametrize("make", [lambda: _cases()["tgv_n8"], _small_sphere],
                         ids=["tgv_n8", "sphere"])
def test_graph_launch_count_equals_eager(precision, method, make):
    """The kernel count a replayed step graph reports (computed from the
    case's tables) equals the count of the same steps launched one by one."""
    case = make()
    counts = []
    for graph in (False, True):
        ctx = api.CaseContext(case, precision=precision)
        ctx.set_method(method)
        ctx.set_state(case.U, case.U, case.U)
        ctx.advance(1, 3, use_graph=graph)
        if graph:  # the first graph call captures; count a replay
            ctx.advance(1, 3, use_graph=True)
        counts.append(ctx.launch_count())
        ctx.close()
    assert counts[0] == counts[1] > 0, counts


@pytest.mark.parametrize("graph", [False, True])
def test_sphere_ibm_two_level_bitwise(port, graph):
    """Sphere with IBM ghost cells on a two-level grid with open-domain
    boundary conditions: every hot-path component in one loop."""
    case = _small_sphere()
    a = O.State(case)
    port.run(case, a, 2, 2)
    ctx = api.CaseContext(case)
    ctx.set_state(case.U, case.U, case.U)
    er = ctx.advance(2, 2, use_graph=graph)
    U1_, U1, U1q = ctx.get_state()
    assert np.array_equal(U1_, a.U1_) and np.array_equal(U1, a.U1) and np.array_equal(U1q, a.U1q)
    assert np.allclose(er[1:6], a.er[1:6], rtol=1e-12, atol=0)
    # force integrals (drag / lift like terms, er[6], er[7])
    scale = np.abs(a.Residual1).max() / (0.5 * case.phys.rho0 * case.phys.U0 ** 2 * 2.602)
    assert abs(er[6] - a.er[6]) <= 1e-12 * max(abs(a.er[6]), scale)
    assert abs(er[7] - a.er[7]) <= 1e-12 * max(abs(a.er[7]), scale)
    ctx.close()


@pytest.mark.parametrize("graph", [False, True])
def test_tile_shape_keeps_fp64_bitwise(port, graph):
    """Tile edge 4 instead of 8: the same per-cell arithmetic, so the FP64
    state after whole dual-time steps still equals the oracle's bit for bit."""
    case = _cases()["two_level_open_n8"]
    a = O.State(case)
    port.run(case, a, G.RUN_STEPS, G.RUN_SUBITERS)
    ctx = api.CaseContext(case)
    ctx.set_tuning(flux_tile=4)
    ctx.set_state(case.U, case.U, case.U)
    er = ctx.advance(G.RUN_STEPS, G.RUN_SUBITERS, use_graph=graph)
    U1_, U1, U1q = ctx.get_state()
    assert np.array_equal(U1_, a.U1_) and np.array_equal(U1, a.U1) and np.array_equal(U1q, a.U1q)
    assert np.allclose(er[1:6], a.er[1:6], rtol=1e-12, atol=0)
    with pytest.raises(api.BcmgError):
        ctx.set_tuning(flux_tile=6)
    ctx.close()


def test_autotune_applies_a_valid_shape(port):
    case = cases.taylor_green(ncx=2, n=16)
    for prec in (api.PRECISION_FP64, api.PRECISION_SPLIT):
        ctx = api.CaseContext(case, precision=prec)
        ctx.set_method(api.METHOD_LUSGS)
        ctx.set_state(case.U, case.U, case.U)
        before = ctx.get_state()
        res = ctx.autotune(2)
        assert res["flux_tile"] in (4, 8)
        assert res["flux_ms"]["8_packed"] > 0 and res["flux_ms"]["4"] > 0
        if prec == api.PRECISION_SPLIT:
            # both split flux forms on 8^3 tiles, and the LU-SGS sweep widths
            assert res["flux_ms"]["8_single"] > 0
            assert res["flux_form"] in ((1, 2) if res["flux_tile"] == 8 else (0,))
            assert res["lusgs_ms"]["widest"] > 0 and res["lusgs_ms"]["half"] > 0
        after = ctx.get_state()  # the tuner restores the state it timed on
        for x, y in zip(before, after):
            assert np.array_equal(x, y)
        ctx.advance(1, 2)
        ctx.close()
