"""The stage entry point that allocates nothing, against the regular one.

bcmg_flux_rk_stage_noalloc serves callers that cannot let a library call
cudaMalloc -- solvers that hand out every device buffer from their own
pre-sized arena, and latency-sensitive hosts that cannot accept the implicit
device synchronisation an allocation may cause.  The caller passes device
buffers for all inputs and outputs; the only scratch (the norm partial sums)
is a static device array shared by every call.  This file is collected last
so that a failure here does not hide the results of the other GPU tests.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from bcm_cgli_gb300 import api, cases
from bcm_cgli_gb300._lib import last_error, lib

pytestmark = pytest.mark.gpu

NORM_RTOL = 1e-12  # same tolerance as the other parity tests for the norm sums
# Arrays each stage writes (RK 1 writes U1p1, RK 2 writes U1p2; RK 3 neither).
WRITTEN = {1: ("U1_", "U1p1", "Rku1", "Residual1"), 2: ("U1_", "U1p2", "Rku1", "Residual1"),
           3: ("U1_", "Rku1", "Residual1")}
ARRAYS = ("U1_", "U1", "U1q", "U1p1", "U1p2", "Rku1", "Residual1")


@pytest.fixture
def reference_config():
    """Restores the twins' default reference configuration afterwards."""
    yield
    api.set_reference_config()


def _entry():
    f = lib().bcmg_flux_rk_stage_noalloc
    f.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double] + [C.c_void_p] * 11
    f.restype = C.c_int
    return f


def _case(seed):
    return cases.random_case(seed=seed, ncx=2, ncy=2, ncz=2, n=8, periodic=True, viscous=True)


def _stage_through_both(torch, case, RK):
    """One stage from the same state through the regular twin (host arrays)
    and through the entry point that allocates nothing (device arrays);
    returns (regular state, device arrays, device er)."""
    dev = torch.device("cuda:0")
    ref = O.State(case)
    api.BCM_Flux_XYZ_Viscous_Runge_kutta(0, case.ncube, RK, case.dT, case.dTau, case.e,
                                         case.fws, case.csl, case.cube_size, ref.U1_, ref.U1,
                                         ref.U1q, ref.U1p1, ref.U1p2, ref.Rku1, ref.Residual1,
                                         ref.er)
    st = O.State(case)
    src = dict(FWS=case.fws, cube_size=case.cube_size, **{k: getattr(st, k) for k in ARRAYS})
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in src.items()}
    er = torch.zeros(8, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    return ref, d, er


def _call(f, torch, case, RK, d, er):
    stream = torch.cuda.current_stream(torch.device("cuda:0")).cuda_stream
    rc = f(case.ncube, RK, case.dT, case.dTau, case.e, d["FWS"].data_ptr(),
           d["cube_size"].data_ptr(), d["U1_"].data_ptr(), d["U1"].data_ptr(),
           d["U1q"].data_ptr(), d["U1p1"].data_ptr(), d["U1p2"].data_ptr(),
           d["Rku1"].data_ptr(), d["Residual1"].data_ptr(), er.data_ptr(), stream)
    assert rc == 0, last_error()
    torch.cuda.synchronize()


@pytest.mark.parametrize("RK", [1, 2, 3])
def test_noalloc_stage_matches_regular_entry_point_on_two_calls(RK, reference_config):
    torch = pytest.importorskip("torch")
    f = _entry()
    # Two calls in a row on different states: the second must not see the
    # first call's scratch contents.
    for seed in (41, 42):
        case = _case(seed)
        api.reference_config_for(case)
        ref, d, er = _stage_through_both(torch, case, RK)
        _call(f, torch, case, RK, d, er)
        # every array bit for bit: the ones the stage writes and the ones it
        # must leave alone
        for k in ARRAYS:
            got = d[k].cpu().numpy()
            assert np.array_equal(got, getattr(ref, k)), (seed, RK, k)
        if RK != 3:
            continue
        e = er.cpu().numpy()
        scale = max(np.abs(ref.Residual1).max(), 1e-300)
        for m in range(1, 8):
            tol = NORM_RTOL * (max(abs(ref.er[m]), 1e-300) if m <= 5 else max(abs(ref.er[m]), scale))
            assert abs(e[m] - ref.er[m]) <= tol, (seed, m, e[m], ref.er[m])


def test_noalloc_call_leaves_free_device_memory_unchanged(reference_config):
    torch = pytest.importorskip("torch")
    f = _entry()
    case = _case(43)
    api.reference_config_for(case)
    ref, d, er = _stage_through_both(torch, case, 3)
    _call(f, torch, case, 3, d, er)  # the first call on the device loads the module
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(3):
        _call(f, torch, case, 3, d, er)
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_cases_beyond_its_scratch(reference_config):
    torch = pytest.importorskip("torch")
    f = _entry()
    api.set_reference_config(ncube_x=32, mpi_ncube=1100)
    buf = torch.zeros(8, dtype=torch.float64, device="cuda:0")
    p = buf.data_ptr()
    # 1100 cubes of 32^3 cells exceed the 33,554,432-cell bound; the call must
    # fail before it launches anything.
    rc = f(1101, 3, 1e-4, 5e-7, 0.1, p, p, p, p, p, p, p, p, p, p, 0)
    assert rc != 0
    assert "scratch" in (last_error() or "")
