"""Split-precision path against the FP64 path (which is bit-exact with the
reference).  Bound: relative L2 error <= 1e-5 per conservative variable
(momentum components relative to the momentum-magnitude norm, since rho*w
of these flows is ~0) after the same steps from the same state."""
import numpy as np
import pytest

from bcm_cgli_gb300 import api, cases
from golden import golden_cases as G

pytestmark = pytest.mark.gpu

SPLIT_BOUND = 1e-5


def rel_l2(a, b, n):
    ai = a[1:, 2:n + 2, 2:n + 2, 2:n + 2].reshape(-1, 5)
    bi = b[1:, 2:n + 2, 2:n + 2, 2:n + 2].reshape(-1, 5)
    d = ai - bi
    mom = np.linalg.norm(bi[:, 1:4])
    return [np.linalg.norm(d[:, 0]) / np.linalg.norm(bi[:, 0])] + \
           [np.linalg.norm(d[:, v]) / mom for v in (1, 2, 3)] + \
           [np.linalg.norm(d[:, 4]) / np.linalg.norm(bi[:, 4])]


def run(case, precision, steps, subiters, graph=True):
    ctx = api.CaseContext(case, precision=precision)
    ctx.set_state(case.U, case.U, case.U)
    er = ctx.advance(steps, subiters, use_graph=graph)
    U = ctx.get_state()
    ctx.close()
    return U, er


@pytest.mark.parametrize("name", sorted(G.golden_cases()))
def test_split_within_bound_of_fp64(name):
    case = G.golden_cases()[name]
    (a, _, _), er_a = run(case, api.PRECISION_FP64, 2, 3)
    (b, _, _), er_b = run(case, api.PRECISION_SPLIT, 2, 3)
    err = rel_l2(b, a, case.n)
    assert max(err) <= SPLIT_BOUND, err
    # the change norms agree to FP32-level relative accuracy where they are
    # not dominated by round-off (components of order 1 after normalisation)
    for m in (1, 2, 3, 5):
        assert abs(er_a[m] - er_b[m]) <= 1e-3 * max(abs(er_a[m]), 1e-12), (m, er_a, er_b)


def test_split_graph_replay_is_identical():
    case = G.golden_cases()["tgv_n8"]
    (a, a1, a2), _ = run(case, api.PRECISION_SPLIT, 2, 2, graph=False)
    (b, b1, b2), _ = run(case, api.PRECISION_SPLIT, 2, 2, graph=True)
    assert np.array_equal(a, b) and np.array_equal(a1, b1) and np.array_equal(a2, b2)


def _prologue_cases():
    cs = dict(G.golden_cases())
    cs["sphere_two_level"] = cases.sphere_ibm(n=8, coarse=2.0, box=((-2, 4), (-2, 2), (-2, 2)),
                                              refine_box=((-2, 2), (-2, 2), (-2, 2)))
    return cs


@pytest.mark.parametrize("name", sorted(_prologue_cases()))
@pytest.mark.parametrize("precision", [api.PRECISION_FP64, api.PRECISION_SPLIT])
def test_reduced_prologue_copies_change_no_cell(name, precision):
    """advance() runs only the face copies that can change a cell in the
    interface call ahead of every stage but a step's first; single stage()
    calls run all of them.  Two sub-iterations both ways end in the same
    state, bit for bit."""
    case = _prologue_cases()[name]
    states = []
    for stepped in (False, True):
        ctx = api.CaseContext(case, precision=precision)
        ctx.set_state(case.U, case.U, case.U)
        if stepped:
            for _ in range(2):
                for RK in (1, 2, 3):
                    ctx.stage(RK)
        else:
            ctx.advance(1, 2, use_graph=False)
        states.append(ctx.get_state()[0])
        ctx.close()
    assert np.array_equal(states[0].view(np.uint64), states[1].view(np.uint64))


@pytest.mark.parametrize("name", sorted(_prologue_cases()))
@pytest.mark.parametrize("graph", [False, True])
def test_face_copies_in_flux_kernel_change_no_cell(name, graph):
    """Split RK stages make the same-level face copies inside the flux kernel
    by default; with the copies left to the interface call after the stage
    the state after two sub-iterations is the same, bit for bit, in every
    cell (ghost layers included)."""
    case = _prologue_cases()[name]
    states = []
    for in_flux in (True, False):
        ctx = api.CaseContext(case, precision=api.PRECISION_SPLIT)
        ctx.set_face_copies(in_flux)
        ctx.set_state(case.U, case.U, case.U)
        ctx.advance(1, 2, use_graph=graph)
        states.append(ctx.get_state())
        ctx.close()
    for a, b in zip(*states):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("name", ["sphere_two_level", "tgv_n8"])
def test_face_copies_in_lusgs_sweep_change_no_cell(name):
    """The split LU-SGS sweep makes the same-level copies of the cells it
    updates as well; with the copies left to the interface call the state is
    the same, bit for bit."""
    case = _prologue_cases()[name]
    states = []
    for in_flux in (True, False):
        ctx = api.CaseContext(case, precision=api.PRECISION_SPLIT)
        ctx.set_method(api.METHOD_LUSGS)
        ctx.set_face_copies(in_flux)
        ctx.set_state(case.U, case.U, case.U)
        ctx.advance(1, 3)
        states.append(ctx.get_state())
        ctx.close()
    for a, b in zip(*states):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_face_copies_in_flux_kernel_batch():
    """The same for a batch (periodic TGV, a random two-level case, the
    two-level sphere with IBM tables), through fixed and convergence-driven
    stepping."""
    cs = [cases.taylor_green(ncx=2, n=8), cases.random_two_level_case(seed=6, n=8, periodic=False),
          _prologue_cases()["sphere_two_level"]]
    out = []
    for in_flux in (True, False):
        bt = api.BatchContext(cs, precision=api.PRECISION_SPLIT)
        bt.set_face_copies(in_flux)
        for q, c in enumerate(cs):
            bt.set_case_state(q, c.U, c.U, c.U)
        bt.advance(1, 2)
        bt.advance_converged(1, 6, tol=0.5)
        out.append([bt.get_case_state(q)[0] for q in range(len(cs))])
        bt.close()
    for a, b in zip(*out):  # cube slot 0 of a case's arrays is not state
        assert np.array_equal(a[1:].view(np.uint64), b[1:].view(np.uint64))


def test_split_vortex_config1_size():
    """Config-1 size (4x4x4 cubes of 16^3, inviscid vortex, M 0.5): 3 dual-time
    steps of 10 sub-iterations, split vs FP64."""
    case = cases.isentropic_vortex(ncx=4, n=16)
    (a, _, _), _ = run(case, api.PRECISION_FP64, 3, 10)
    (b, _, _), _ = run(case, api.PRECISION_SPLIT, 3, 10)
    err = rel_l2(b, a, case.n)
    assert max(err) <= SPLIT_BOUND, err


def test_split_sphere_forces_within_bound():
    """Sphere IBM case: split state within the bound and the drag/lift
    integrals (er[6], er[7]) within 0.1% of the FP64 path."""
    case = cases.sphere_ibm(n=8, coarse=2.0, box=((-2, 4), (-2, 2), (-2, 2)),
                            refine_box=((-2, 2), (-2, 2), (-2, 2)))
    (a, _, _), er_a = run(case, api.PRECISION_FP64, 2, 3)
    (b, _, _), er_b = run(case, api.PRECISION_SPLIT, 2, 3)
    err = rel_l2(b, a, case.n)
    assert max(err) <= SPLIT_BOUND, err
    assert abs(er_b[6] - er_a[6]) <= 1e-3 * abs(er_a[6]), (er_a[6], er_b[6])


@pytest.mark.parametrize("workload", ["tgv", "sphere", "batch"])
def test_split_full_size_within_bound(workload):
    """Benchmark sizes (config 2 TGV 7.1 M cells, config 3 sphere 6.5 M cells
    with the GPU-built IBM tables, config 4 batch of 16 spheres): one
    dual-time step of 10 sub-iterations, split against FP64 within 1e-5
    relative L2 per variable, and every case's drag within 0.1%."""
    if workload == "tgv":
        cs = [cases.taylor_green(ncx=8, n=24)]
    elif workload == "sphere":
        cs = [cases.sphere_ibm(preprocess=api.ibm_preprocess)]
    else:
        cs = cases.sphere_batch(ncase=16, seed=2024, n=16, preprocess=api.ibm_preprocess)
    states, ers = {}, {}
    for prec in (api.PRECISION_FP64, api.PRECISION_SPLIT):
        ctx = (api.BatchContext(cs, precision=prec) if len(cs) > 1
               else api.CaseContext(cs[0], precision=prec))
        if len(cs) > 1:
            for q, c in enumerate(cs):
                ctx.set_case_state(q, c.U, c.U, c.U)
        else:
            ctx.set_state(cs[0].U, cs[0].U, cs[0].U)
        er = ctx.advance(1, 10)
        states[prec] = ([ctx.get_case_state(q)[0] for q in range(len(cs))] if len(cs) > 1
                        else [ctx.get_state()[0]])
        ers[prec] = np.asarray(er).reshape(len(cs), 8)
        ctx.close()
    for q, c in enumerate(cs):
        err = rel_l2(states[api.PRECISION_SPLIT][q], states[api.PRECISION_FP64][q], c.n)
        assert max(err) <= SPLIT_BOUND, (q, err)
        if workload != "tgv":
            a, b = ers[api.PRECISION_FP64][q, 6], ers[api.PRECISION_SPLIT][q, 6]
            assert abs(b - a) <= 1e-3 * abs(a), (q, a, b)


def _mirror_ref(U, rho0, P0):
    d = U.copy()
    d[..., 0] -= rho0
    d[..., 4] -= P0 / (1.4 - 1)
    return d.astype(np.float32)  # IEEE round to nearest even


def test_mirror_is_the_ieee_rounding_of_the_deltas():
    """The FP32 mirror (formed with an integer round-to-nearest-even
    conversion) equals numpy's IEEE conversion of the FP64 deltas, bit for
    bit, for values spread over many binades and for per-case reference
    states in a batch."""
    a = cases.random_case(seed=31, n=8, periodic=True)
    b = cases.random_case(seed=32, n=8, periodic=False)
    b.phys.rho0, b.phys.P0 = 0.93, 87000.0
    rng = np.random.default_rng(5)
    for c in (a, b):  # momentum spread over many binades, some exact zeros
        c.U[..., 2] *= 10.0 ** rng.integers(-12, 6, size=c.U.shape[:-1])
        c.U[..., 3][rng.random(c.U.shape[:-1]) < 0.05] = 0.0
    ctx = api.CaseContext(a, precision=api.PRECISION_SPLIT)
    ctx.set_state(a.U, a.U, a.U)
    M = ctx.mirror()
    ref = _mirror_ref(a.U, a.phys.rho0, a.phys.P0)
    assert np.array_equal(M[1:].view(np.uint32), ref[1:].view(np.uint32))
    ctx.close()
    bt = api.BatchContext([a, b], precision=api.PRECISION_SPLIT)
    for q, c in enumerate((a, b)):
        bt.set_case_state(q, c.U, c.U, c.U)
    M = bt.mirror()
    g = 1
    for c in (a, b):
        ref = _mirror_ref(c.U, c.phys.rho0, c.phys.P0)[1:]
        assert np.array_equal(M[g:g + c.ncube - 1].view(np.uint32), ref.view(np.uint32))
        g += c.ncube - 1
    bt.close()


def _assert_same_bits(M, ref):
    bad = np.argwhere(M[1:].view(np.uint32) != ref[1:].view(np.uint32))
    assert bad.size == 0, (f"{len(bad)} mirror values differ from the state's rounding; "
                           f"first (cube-1, i, j, k, v): {bad[:6].tolist()}")


def _state_mirror(U, members):
    """numpy's IEEE rounding of the state's deltas, per case of a batch."""
    out = np.empty(U.shape, np.float32)
    g = 1
    for c in members:
        m = c.ncube - 1
        out[g:g + m] = _mirror_ref(U[g:g + m], c.phys.rho0, c.phys.P0)
        g += m
    return out


@pytest.mark.parametrize("name", sorted(_prologue_cases()))
@pytest.mark.parametrize("method", ["rk3", "lusgs"])
def test_kept_mirror_is_the_rounding_of_the_state(name, method):
    """The mirror the kernels keep during stepping (one full pass per
    dual-time step; the flux kernel, interface, boundary and IBM kernels and
    the LU-SGS sweep write the values of the cells they change) equals the
    IEEE rounding of the state in every cell after single stages, eager and
    graph steps, and the state equals the one obtained with a full mirror
    pass before every flux launch, bit for bit."""
    case = _prologue_cases()[name]
    states = []
    for each_stage in (False, True):
        ctx = api.CaseContext(case, precision=api.PRECISION_SPLIT)
        if method == "lusgs":
            ctx.set_method(api.METHOD_LUSGS)
        ctx.set_mirror_each_stage(each_stage)
        ctx.set_state(case.U, case.U, case.U)
        if method == "rk3":
            ctx.stage(1)
            ctx.stage(2)
        ctx.advance(1, 2, use_graph=False)
        ctx.advance(2, 2, use_graph=True)
        U = ctx.get_state()
        if not each_stage:
            M = ctx.mirror_current()
            ref = _state_mirror(U[0], [case])
            _assert_same_bits(M, ref)
        states.append(U)
        ctx.close()
    for a, b in zip(*states):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_kept_mirror_batch_with_converged_cases():
    """A batch whose cases converge at different sub-iterations (converged
    cases sit out the rest of the step, then rejoin at the next): the kept
    mirror still equals the rounding of the state, and the states equal
    those of a full mirror pass before every flux launch."""
    cs = [cases.taylor_green(ncx=2, n=8), cases.random_two_level_case(seed=6, n=8, periodic=False),
          _prologue_cases()["sphere_two_level"]]
    out = []
    for each_stage in (False, True):
        bt = api.BatchContext(cs, precision=api.PRECISION_SPLIT)
        bt.set_mirror_each_stage(each_stage)
        for q, c in enumerate(cs):
            bt.set_case_state(q, c.U, c.U, c.U)
        bt.advance(1, 2)
        _, its = bt.advance_converged(2, 7, tol=0.5)
        bt.advance(1, 1)
        U = bt.get_state()[0]
        if not each_stage:
            M = bt.mirror_current()
            _assert_same_bits(M, _state_mirror(U, cs))
        out.append(U)
        bt.close()
    assert np.array_equal(out[0][1:].view(np.uint64), out[1][1:].view(np.uint64))
