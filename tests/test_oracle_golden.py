"""Pin the oracle (the C restatement in oracle/bcm_oracle.c) against the
reference's own outputs: digests recorded by tests/golden/make_golden.py
from the reference's compiled sources, and, where the reference sources are
present, a direct bit-for-bit comparison on more random cases."""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle as O
from golden import golden_cases as G

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = json.load(open(os.path.join(HERE, "golden", "golden.json")))


def digest(a):
    return hashlib.sha256(G.canonical(a)).hexdigest()


@pytest.fixture(scope="module")
def port():
    p = O.Port()
    p.set_threads(4)
    return p


@pytest.mark.parametrize("name", sorted(GOLD["cases"]))
def test_routines_match_reference_digests(port, name):
    case = G.golden_cases()[name]
    rec = GOLD["cases"][name]
    for r, fn in (("bc", lambda s: port.bc(case, s.U1_)),
                  ("ghost_minus", lambda s: port.ghost(case, s.U1_, -1)),
                  ("ghost_plus", lambda s: port.ghost(case, s.U1_, 1)),
                  ("interface", lambda s: port.interface(case, s.U1_))):
        st = O.State(case)
        fn(st)
        assert digest(st.U1_) == rec[r], f"{name}: {r} differs from the reference"
    st = O.State(case)
    for RK in (1, 2, 3):
        port.flux_stage(case, st, RK)
        for k, d in rec[f"flux{RK}"].items():
            assert digest(getattr(st, k)) == d, f"{name}: flux stage {RK} {k}"
    assert [repr(float(x)) for x in st.er] == rec["flux3_er"]


@pytest.mark.parametrize("name", sorted(GOLD["cases"]))
def test_full_loop_matches_reference_digests(port, name):
    case = G.golden_cases()[name]
    rec = GOLD["cases"][name]
    st = O.State(case)
    port.run(case, st, GOLD["steps"], GOLD["subiters"])
    for k, d in rec["run"].items():
        assert digest(getattr(st, k)) == d, f"{name}: run {k}"
    assert [repr(float(x)) for x in st.er] == rec["run_er"]
    assert [repr(float(x)) for x in st.Emax] == rec["run_emax"]


def _direct_cases():
    """Random 2x2x2 boxes, and the degenerate grids: one periodic cube (each
    face its own neighbour), a 3x2x2 open box (boundary faces on every side,
    cubes with one neighbour along an axis) and a case without IBM tables."""
    from bcm_cgli_gb300 import cases
    out = {f"random_{s}": (lambda s=s: cases.random_case(seed=s, n=4, periodic=bool(s % 2),
                                                         viscous=True)) for s in (21, 22, 23)}
    out["one_cube_periodic"] = lambda: cases.random_case(seed=24, ncx=1, ncy=1, ncz=1, n=4,
                                                         periodic=True)
    out["open_3x2x2"] = lambda: cases.random_case(seed=25, ncx=3, ncy=2, ncz=2, n=4,
                                                  periodic=False)
    out["no_ibm"] = lambda: cases.random_case(seed=26, n=4, periodic=False, with_ibm=False)
    return out


@pytest.mark.skipif(not O.reference_available(), reason="reference sources not on this host")
@pytest.mark.parametrize("name", list(_direct_cases()))
def test_port_equals_reference_directly(port, name):
    case = _direct_cases()[name]()
    ref = O.Ref(case)
    ref.set_threads(1)
    a, b = O.State(case), O.State(case)
    port.run(case, a, 1, 2)
    ref.run(case, b, 1, 2)
    for k in ("U1_", "U1", "U1q", "Rku1", "Residual1", "U1p1", "U1p2"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert np.array_equal(a.er, b.er)


def test_oracle_thread_count_invariant():
    """The restatement's results do not depend on its thread count (its
    order-sensitive sums are serial), unlike the reference's racy norms."""
    from bcm_cgli_gb300 import cases
    case = cases.random_case(seed=5, n=4)
    p = O.Port()
    out = []
    for t in (1, 3):
        p.set_threads(t)
        st = O.State(case)
        p.run(case, st, 1, 1)
        out.append((st.U1_.copy(), st.er.copy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("name", sorted(GOLD["cases"]))
def test_plot3d_restatement_matches_reference_writer(port, name):
    """oracle/plot3d.py reproduces the bytes of the reference's BCM_Output
    (grid and solution files of the final state of the golden run)."""
    import plot3d
    case = G.golden_cases()[name]
    rec = GOLD["cases"][name]
    st = O.State(case)
    port.run(case, st, GOLD["steps"], GOLD["subiters"])
    x = plot3d.grid_bytes(case.n, case.ncube, case.cube_size, case.origin, case.phys.mpi_ncube)
    q = plot3d.solution_bytes(case.n, st.U1_, case.phys.mpi_ncube)
    assert hashlib.sha256(x).hexdigest() == rec["plot3d_x"]
    assert hashlib.sha256(q).hexdigest() == rec["plot3d_q"]


@pytest.mark.skipif(not O.reference_available(), reason="reference sources not present")
def test_plot3d_restatement_equals_reference_writer_directly(tmp_path):
    """A larger two-level case through the reference's own BCM_Output."""
    import plot3d
    from bcm_cgli_gb300 import cases
    case = cases.random_two_level_case(seed=21, n=8, periodic=False)
    ref = O.Ref(case)
    ref.output(case, case.U.copy(), 12, str(tmp_path))
    x = (tmp_path / "BCMdata00001.x").read_bytes()
    q = (tmp_path / "qBCMdata00012.q").read_bytes()
    assert x == plot3d.grid_bytes(case.n, case.ncube, case.cube_size, case.origin,
                                  case.phys.mpi_ncube)
    assert q == plot3d.solution_bytes(case.n, case.U, case.phys.mpi_ncube)


@pytest.mark.parametrize("velocity", [(1.0, 0.0, 0.0), (0.6, -0.3, 0.45)])
@pytest.mark.parametrize("make", [lambda: G.golden_cases()["tgv_n8"],
                                  lambda: G.golden_cases()["vortex_n8"]],
                         ids=["viscous", "inviscid"])
def test_free_stream_is_preserved_exactly(port, velocity, make):
    """Known answer: a uniform flow on an all-fluid periodic box stays
    uniform through whole dual-time steps, with or without viscosity and
    for any flow direction, to a few units in the last place: the
    reference's BDF2 source of a state constant in time,
    -(3 Q - 4 Q + Q) / (2 dT), is the rounding error of 3 Q rather than
    exactly zero, so every cell takes a tiny increment (measured: at most
    1 ulp of density and energy after two steps)."""
    case = make()
    ph = case.phys
    speed = ph.U0
    u = [speed * c for c in velocity]
    rho, P = ph.rho0, ph.P0
    q = np.array([rho, rho * u[0], rho * u[1], rho * u[2],
                  P / 0.4 + 0.5 * rho * (u[0] ** 2 + u[1] ** 2 + u[2] ** 2)])
    assert (case.fws == 1).all()
    case.U = np.broadcast_to(q, case.U.shape).copy()
    a = O.State(case)
    port.run(case, a, 2, 2)
    n = case.n
    inner = a.U1_[1:, 2:n + 2, 2:n + 2, 2:n + 2]
    tol = 4 * np.spacing(np.abs(q))  # zero components must stay exactly zero
    assert (np.abs(inner - q) <= tol).all(), np.abs(inner - q).max(axis=(0, 1, 2, 3))
