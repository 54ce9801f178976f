"""The drop-in twins' host-array handling and split-precision option.

* Page-locking the caller's arrays and, with the scratch-kept option, the
  once-per-array upload of the flux twin's write-only arrays change no bit:
  every array equals the oracle's after whole sub-iterations in main.cpp's
  call order (main.cpp:1161-1241).
* The split-precision flux twin stays within 1e-5 relative L2 of the FP64
  twin and leaves U1p1 / U1p2 as the reference's stage combination does
  (the new state of the fluid cells).
"""
import numpy as np
import pytest

import oracle as O
from bcm_cgli_gb300 import api, cases
from golden import golden_cases as G

pytestmark = pytest.mark.gpu

SPLIT_BOUND = 1e-5
ARRAYS = ("U1_", "U1", "U1q", "U1p1", "U1p2", "Rku1", "Residual1")


@pytest.fixture
def twin_defaults():
    """Restores the twins' defaults afterwards."""
    yield
    api.set_reference_precision(api.PRECISION_FP64)
    api.set_twin_scratch_kept(False)
    api.set_host_pinning(False)
    api.set_reference_config()


def _subiteration_twins(case, st):
    """One sub-iteration through the twins in main.cpp's order."""
    xl, xu, yl, yu, zl, zu = (api._one_based(x) for x in case.bc_lists())
    for RK in (1, 2, 3):
        api.BCM_X_boundary_condition(0, len(xl) - 1, len(xu) - 1, xl, xu, st.U1_)
        api.BCM_Y_boundary_condition(len(yl) - 1, len(yu) - 1, yl, yu, st.U1_)
        api.BCM_Z_boundary_condition(len(zl) - 1, len(zu) - 1, zl, zu, st.U1_)
        for which, t in ((-1, case.ibm_minus), (1, case.ibm_plus)):
            if t is None:
                continue
            W, Gi, I = t
            f = api.BCM_Ghostcell_minus if which < 0 else api.BCM_Ghostcell_plus
            f(0, (len(Gi) - 1) // 4, W, Gi, I, case.fws, st.U1_)
        api.BCM_Interface_for_case(case, st.U1_)
        api.BCM_Flux_XYZ_Viscous_Runge_kutta(0, case.ncube, RK, case.dT, case.dTau, case.e,
                                             case.fws, case.csl, case.cube_size, st.U1_,
                                             st.U1, st.U1q, st.U1p1, st.U1p2, st.Rku1,
                                             st.Residual1, st.er)
        api.BCM_Interface_for_case(case, st.U1_)


def _oracle_subiteration(port, case, st):
    for RK in (1, 2, 3):
        port.bc(case, st.U1_)
        port.ghost(case, st.U1_, -1)
        port.ghost(case, st.U1_, 1)
        port.interface(case, st.U1_)
        port.flux_stage(case, st, RK)
        port.interface(case, st.U1_)


@pytest.mark.parametrize("name", ["random_open_n4", "two_level_open_n8", "tgv_n8"])
@pytest.mark.parametrize("mode", ["pinned", "pinned_scratch_kept", "pageable"])
def test_twin_subiterations_bitwise_in_every_copy_mode(name, mode, twin_defaults):
    case = G.golden_cases()[name]
    api.reference_config_for(case)
    api.set_host_pinning(mode != "pageable")
    api.set_twin_scratch_kept(mode == "pinned_scratch_kept")
    port = O.Port()
    a, b = O.State(case), O.State(case)
    for _ in range(2):
        _oracle_subiteration(port, case, a)
        _subiteration_twins(case, b)
    api.release_host_arrays()  # while the arrays are alive
    for k in ARRAYS:
        assert np.array_equal(getattr(a, k), getattr(b, k)), (name, mode, k)


def _packed_state(case):
    """The run's seven arrays side by side in one buffer, each starting 16
    bytes past the previous one's end (so neighbours share pages, as heap
    arrays of a few hundred KB do)."""
    st = O.State(case)
    shape, cnt = st.U1_.shape, st.U1_.size
    buf = np.zeros(len(ARRAYS) * (cnt + 2) + 1, np.float64)
    for m, k in enumerate(ARRAYS):
        v = buf[1 + m * (cnt + 2):1 + m * (cnt + 2) + cnt].reshape(shape)
        v[...] = getattr(st, k)
        setattr(st, k, v)
    return st, buf


@pytest.mark.parametrize("mode", ["pinned", "pinned_scratch_kept", "pageable"])
def test_twin_arrays_sharing_pages(mode, twin_defaults):
    """Caller arrays that share pages with each other: page-locking registers
    only each array's whole pages, so a neighbour starting on a shared page
    is never taken for page-locked memory, and every array still equals the
    oracle's."""
    case = G.golden_cases()["random_open_n4"]
    api.reference_config_for(case)
    api.set_host_pinning(mode != "pageable")
    api.set_twin_scratch_kept(mode == "pinned_scratch_kept")
    port = O.Port()
    a = O.State(case)
    b, buf = _packed_state(case)
    for _ in range(2):
        _oracle_subiteration(port, case, a)
        _subiteration_twins(case, b)
    api.release_host_arrays()  # while the arrays are alive
    for k in ARRAYS:
        assert np.array_equal(getattr(a, k), getattr(b, k)), (mode, k)
    del buf


def test_twins_follow_a_new_cube_size_with_the_same_cube_count(twin_defaults):
    """A case of 8 cubes of 8^3 and then one of 8 cubes of 4^3: the twins
    size their device arrays for the new configuration (the boundary twin,
    called first, must not leave the flux twin the old cell count), copy
    exactly the new arrays, and equal the oracle; the arrays sit in one
    buffer between guard values that must stay untouched."""
    port = O.Port()
    for name in ("tgv_n8", "random_open_n4"):
        case = G.golden_cases()[name]
        api.reference_config_for(case)
        api.set_host_pinning(True)
        a = O.State(case)
        b, buf = _packed_state(case)
        # guards: before the first array, and the two values after each array
        guards = [0] + [i for m in range(len(ARRAYS))
                        for i in (1 + m * (case.U.size + 2) + case.U.size,
                                  2 + m * (case.U.size + 2) + case.U.size)]
        assert guards[-1] == len(buf) - 1
        buf[guards] = -777.0
        _oracle_subiteration(port, case, a)
        _subiteration_twins(case, b)
        api.release_host_arrays()  # while the arrays are alive
        for k in ARRAYS:
            assert np.array_equal(getattr(a, k), getattr(b, k)), (name, k)
        assert np.all(buf[guards] == -777.0), name
        del buf


@pytest.mark.parametrize("name", ["random_periodic_n8", "tgv_n8", "vortex_n8"])
def test_split_flux_twin_within_bound(name, twin_defaults):
    case = G.golden_cases()[name]
    api.reference_config_for(case)
    fp, sp = O.State(case), O.State(case)
    for _ in range(2):
        _subiteration_twins(case, fp)
    api.set_reference_precision(api.PRECISION_SPLIT)
    for _ in range(2):
        _subiteration_twins(case, sp)
    n = case.n
    a = fp.U1_[1:, 2:n + 2, 2:n + 2, 2:n + 2].reshape(-1, 5)
    b = sp.U1_[1:, 2:n + 2, 2:n + 2, 2:n + 2].reshape(-1, 5)
    mom = np.linalg.norm(a[:, 1:4])
    err = [np.linalg.norm(b[:, 0] - a[:, 0]) / np.linalg.norm(a[:, 0])] + \
          [np.linalg.norm(b[:, v] - a[:, v]) / mom for v in (1, 2, 3)] + \
          [np.linalg.norm(b[:, 4] - a[:, 4]) / np.linalg.norm(a[:, 4])]
    assert max(err) <= SPLIT_BOUND, err
    # RK 1 of a further stage: U1p1 holds the new state of the fluid cells
    st = O.State(case)
    st.U1_[...] = sp.U1_
    api.BCM_Flux_XYZ_Viscous_Runge_kutta(0, case.ncube, 1, case.dT, case.dTau, case.e, case.fws,
                                         case.csl, case.cube_size, st.U1_, st.U1, st.U1q,
                                         st.U1p1, st.U1p2, st.Rku1, st.Residual1, st.er)
    fl = case.fws == 1
    fl[:, :2] = fl[:, -2:] = False
    fl[:, :, :2] = fl[:, :, -2:] = False
    fl[:, :, :, :2] = fl[:, :, :, -2:] = False
    fl[0] = False
    assert np.array_equal(st.U1p1[fl], st.U1_[fl])
