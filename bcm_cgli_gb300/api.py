"""Python mirror of the reference's hot-path interface, on the GPU library.

Two layers, matching ``include/bcm_gb300.h``:

* Reference-named functions (``BCM_Flux_XYZ_Viscous_Runge_kutta``,
  ``BCM_X_boundary_condition``, ... ``BCM_Interface``) that take numpy arrays
  in the reference layout and update them in place, with the reference's
  argument order and meaning (``main.h:224-513``).  The reference's
  compile-time ``Resolution.h``/``prm.h`` values are set with
  :func:`set_reference_config`.
* :class:`CaseContext`, the device-resident path: state stays in HBM and
  whole dual-time steps run per call.

Every call goes to the CUDA library; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib, cases
from ._lib import BcmgError, check, lib

PRECISION_FP64 = 0
PRECISION_SPLIT = 1
METHOD_RK3 = 0  # the reference's preconditioned three-stage RK (bit-exact)
METHOD_LUSGS = 1  # LU-SGS sub-iterations (no reference counterpart)


def _dp(a):
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise BcmgError("expected a C-contiguous float64 array")
    return a


def _ip(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a if a.size else np.zeros(1, np.int32)


def _raise_if_failed(name):
    err = _lib.last_error()
    if err:
        raise BcmgError(f"{name}: {err}")


# ---------------------------------------------------------------------------
# Reference compile-time configuration
# ---------------------------------------------------------------------------
def set_reference_config(ncube_x=16, mpi_ncube=1150, mu_L=0.0000185, rho0=1.1842, U0=38.889,
                         Uin=38.889, P0=101300.0):
    """Resolution.h / prm.h values the reference-named functions use."""
    cfg = _lib.RefConfig(ncube_x, mpi_ncube, mu_L, rho0, U0, Uin, P0)
    check(lib().bcmg_set_reference_config(C.byref(cfg)))


def reference_config_for(case):
    ph = case.phys
    set_reference_config(case.n, ph.mpi_ncube, ph.mu_L, ph.rho0, ph.U0, ph.Uin, ph.P0)


def set_reference_precision(precision):
    """Arithmetic of the BCM_Flux_XYZ_Viscous_Runge_kutta twin:
    PRECISION_FP64 (default, bit-identical to the reference) or
    PRECISION_SPLIT (the stage update inside the flux kernel; Rku1 is not
    written)."""
    check(lib().bcmg_set_reference_precision(int(precision)))


def release_host_arrays():
    """Unregisters every host array the twins page-locked and forgets them
    (before freeing an array the twins have seen)."""
    lib().bcmg_release_host_arrays()


def set_host_pinning(on=True):
    """Whether the twins page-lock the caller's arrays (default off).  With it
    on, call release_host_arrays() before any array the twins have seen is
    freed."""
    lib().bcmg_set_host_pinning(1 if on else 0)


def set_twin_scratch_kept(on=True):
    """The flux twin uploads its write-only scratch arrays (U1p1 at RK 1,
    U1p2 at RK 2, Rku1, Residual1 at RK 1 and 2) once per host array instead
    of every call: for callers that change them only through the twins."""
    lib().bcmg_set_twin_scratch_kept(1 if on else 0)


# ---------------------------------------------------------------------------
# Reference-named entry points (in place on host arrays)
# ---------------------------------------------------------------------------
def BCM_Flux_XYZ_Viscous_Runge_kutta(myid, ncube, RK, deltaT, deltaTau, e, FWS, csl, cube_size,
                                     U1_, U1, U1q, U1p1, U1p2, Rku1, Residual1, er):
    lib().BCM_Flux_XYZ_Viscous_Runge_kutta(
        int(myid), int(ncube), int(RK), float(deltaT), float(deltaTau), float(e), _ip(FWS),
        _ip(csl), _dp(cube_size), _dp(U1_), _dp(U1), _dp(U1q), _dp(U1p1), _dp(U1p2), _dp(Rku1),
        _dp(Residual1), _dp(er))
    _raise_if_failed("BCM_Flux_XYZ_Viscous_Runge_kutta")


def _one_based(lst):
    return np.concatenate([np.zeros(1, np.int32), np.asarray(lst, np.int32)])


def BCM_X_boundary_condition(myid, nXbc_l, nXbc_u, Xbc_l, Xbc_u, U1_):
    lib().BCM_X_boundary_condition(int(myid), int(nXbc_l), int(nXbc_u), _ip(Xbc_l),
                                   _ip(Xbc_u), _dp(U1_))
    _raise_if_failed("BCM_X_boundary_condition")


def BCM_Y_boundary_condition(nYbc_l, nYbc_u, Ybc_l, Ybc_u, U1_):
    lib().BCM_Y_boundary_condition(int(nYbc_l), int(nYbc_u), _ip(Ybc_l), _ip(Ybc_u), _dp(U1_))
    _raise_if_failed("BCM_Y_boundary_condition")


def BCM_Z_boundary_condition(nZbc_l, nZbc_u, Zbc_l, Zbc_u, U1_):
    lib().BCM_Z_boundary_condition(int(nZbc_l), int(nZbc_u), _ip(Zbc_l), _ip(Zbc_u), _dp(U1_))
    _raise_if_failed("BCM_Z_boundary_condition")


def BCM_Ghostcell_minus(myid, NNBC, weight, GCindex, IPsur, FWS, U1_):
    n = C.c_int(int(NNBC))
    lib().BCM_Ghostcell_minus(int(myid), C.byref(n), _dp(weight), _ip(GCindex), _ip(IPsur),
                              _ip(FWS), _dp(U1_))
    _raise_if_failed("BCM_Ghostcell_minus")


def BCM_Ghostcell_plus(myid, NNBC, weight, GCindex, IPsur, FWS, U1_):
    n = C.c_int(int(NNBC))
    lib().BCM_Ghostcell_plus(int(myid), C.byref(n), _dp(weight), _ip(GCindex), _ip(IPsur),
                             _ip(FWS), _dp(U1_))
    _raise_if_failed("BCM_Ghostcell_plus")


def _fws_inplace(FWS):
    if FWS.dtype != np.int32 or not FWS.flags.c_contiguous:
        raise BcmgError("FWS must be a C-contiguous int32 array (updated in place)")
    return FWS


def BCM_Immersed_boundary(myid, ncube, n_wallcube, NBC, Xmin, Xmax, Ymin, Ymax, Zmin, Zmax,
                          cube_size, csl, Xcube, Ycube, Zcube, Xcnt, Ycnt, Zcnt, FWS, wallcube):
    """BCM_Immersed_boundary.cpp:127-1081 on the GPU: reads BCM_STL_fine.stl
    in the working directory, updates FWS in place and writes
    IBM_minus<myid>.dat / IBM_plus<myid>.dat.  Xcnt/Ycnt/Zcnt may be None
    (centres formed from the cube corners).  NBC, n_wallcube, the domain
    bounds and wallcube are unused, as in the reference."""
    cen = [None if a is None else _dp(a) for a in (Xcnt, Ycnt, Zcnt)]
    lib().BCM_Immersed_boundary(int(myid), int(ncube), int(n_wallcube), None, float(Xmin),
                                float(Xmax), float(Ymin), float(Ymax), float(Zmin), float(Zmax),
                                _dp(cube_size), _ip(csl), _dp(Xcube), _dp(Ycube), _dp(Zcube),
                                *(None if a is None else a.ctypes.data for a in cen),
                                _fws_inplace(FWS), None)
    _raise_if_failed("BCM_Immersed_boundary")


def ibm_preprocess(case, tris, fws=None):
    """The IBM preprocessing of BCM_Immersed_boundary in memory, on the GPU:
    tris[ntri, 3, 3] in STL facet order; fws (default case.fws) updated in
    place.  Returns the minus and plus tables, each (GCindex[m,4],
    IPsur[m,4], weight[m,8]) with 0-based rows and unrounded weights."""
    fws = _fws_inplace(case.fws if fws is None else fws)
    tri = np.ascontiguousarray(np.asarray(tris, np.float64).reshape(-1, 9))
    cap = int((fws == 0).sum()) + 1
    o = np.ascontiguousarray(case.origin, dtype=np.float64)
    out = [np.zeros(4 * cap, np.int32), np.zeros(4 * cap, np.int32), np.zeros(8 * cap),
           np.zeros(4 * cap, np.int32), np.zeros(4 * cap, np.int32), np.zeros(8 * cap)]
    nm, npl = C.c_int(), C.c_int()
    check(lib().bcmg_ibm_preprocess(
        int(case.n), int(case.ncube), np.ascontiguousarray(case.cube_size, np.float64),
        _ip(case.csl), np.ascontiguousarray(o[:, 0]), np.ascontiguousarray(o[:, 1]),
        np.ascontiguousarray(o[:, 2]), fws, tri.shape[0], tri if tri.size else np.zeros(9),
        cap, C.byref(nm), out[0], out[1], out[2], C.byref(npl), out[3], out[4], out[5]))
    m, p = nm.value, npl.value
    return ((out[0][:4 * m].reshape(m, 4), out[1][:4 * m].reshape(m, 4),
             out[2][:8 * m].reshape(m, 8)),
            (out[3][:4 * p].reshape(p, 4), out[4][:4 * p].reshape(p, 4),
             out[5][:8 * p].reshape(p, 8)))


def interface_lists(case):
    """The 15 neighbour lists of BCM_Interface_table.cpp:96-308 (1-based
    arrays): per axis x, y, z the same-level, big->small (+), small->big (+),
    big->small (-) and small->big (-) lists."""
    adj, csl = case.adj, case.csl
    out = []
    for ax in range(3):
        eq, bsp, sbp, bsm, sbm = [], [], [], [], []
        for c in range(1, case.ncube):
            plus = adj[c, 1:5, 2 + 2 * ax]
            if (plus > 0).any():
                a = plus.max()
                (eq if csl[c] == csl[a] else (sbp if csl[c] < csl[a] else bsp)).append(c)
            minus = adj[c, 1:5, 1 + 2 * ax]
            if (minus > 0).any():
                a = minus.max()
                if csl[c] < csl[a]:
                    sbm.append(c)
                elif csl[c] > csl[a]:
                    bsm.append(c)
        out.append([_one_based(x) for x in (eq, bsp, sbp, bsm, sbm)])
    return out


def BCM_Interface_for_case(case, U1_):
    """BCM_Interface with single-process (empty exchange) arguments, like the
    reference's call at main.cpp:1177-1204 on one rank."""
    L = lib()
    lists = interface_lists(case)
    z = np.zeros(4, np.int32)
    d = np.zeros(4)
    zp = z.ctypes.data_as(C.c_void_p)
    dd = d.ctypes.data_as(C.c_void_p)
    adj = np.ascontiguousarray(case.adj, np.int32)
    csl = np.ascontiguousarray(case.csl, np.int32)
    U = _dp(U1_)
    cnt = lambda a: C.c_int(len(a) - 1)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)
    X, Y, Z = lists
    args = ([C.c_int(0), C.c_int(case.ncube), C.c_int(1), C.c_int(0), C.c_int(0), C.c_int(0),
             C.c_int(0), C.c_int(0), C.c_int(0), cnt(X[0]), cnt(Y[0]), cnt(Z[0])] +
            [cnt(a) for a in X[1:] + Y[1:] + Z[1:]] +
            [zp] * 15 + [dd] * 4 + [zp] * 4 + [dd] * 4 + [zp] * 4 + [dd] * 4 + [zp] * 8 +
            [ptr(csl), ptr(adj), ptr(X[0]), ptr(Y[0]), ptr(Z[0])] +
            [ptr(a) for a in X[1:] + Y[1:] + Z[1:]] + [ptr(U)])
    assert len(args) == 85
    L.BCM_Interface(*args)
    _raise_if_failed("BCM_Interface")


def BCM_FWS_Interface(myid, ncube, mPI_Nadj, ncpu_eq, max_nei_eq, nadjX_eq, nadjY_eq, nadjZ_eq,
                      csl, adj_number, adjX_eq, adjY_eq, adjZ_eq, FWS):
    """BCM_FWS_Interface (BCM_FWS_Interface.cpp:23-791, setup, on the host) on
    one process: same-level ghost-face copies of the flags, sign threshold
    and hole fill of every finest-level cube, FWS updated in place.  The
    exchange arguments of main.h:55-110 between nadjZ_eq and csl are passed
    as empty; ncpu_eq must be 0.  adjX/Y/Z_eq are 1-based lists as
    BCM_Interface_table builds them."""
    z = np.zeros(4, np.int32)
    d = np.zeros(4)
    zp, dd = z.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p)
    lists = [_ip(a) for a in (adjX_eq, adjY_eq, adjZ_eq)]
    lib().BCM_FWS_Interface(int(myid), int(ncube), int(mPI_Nadj), int(ncpu_eq), int(max_nei_eq),
                            int(nadjX_eq), int(nadjY_eq), int(nadjZ_eq), *([zp] * 11),
                            *([dd] * 4), *([zp] * 3), _ip(csl), _ip(adj_number),
                            *(a.ctypes.data_as(C.c_void_p) for a in lists), _fws_inplace(FWS))
    _raise_if_failed("BCM_FWS_Interface")


def BCM_FWS_Interface_for_case(case, FWS):
    """BCM_FWS_Interface with the case's same-level lists (interface_lists)
    and single-process arguments, like main.cpp:634 on one rank."""
    X, Y, Z = (lst[0] for lst in interface_lists(case))
    BCM_FWS_Interface(0, case.ncube, 1, 0, 0, len(X) - 1, len(Y) - 1, len(Z) - 1, case.csl,
                      case.adj, X, Y, Z, FWS)


def fws_interface(n, ncube, csl, adj_number, FWS):
    """bcmg_fws_interface: BCM_FWS_Interface for any cube edge n, with the
    same-level pairs found from adj_number; FWS updated in place."""
    if lib().bcmg_fws_interface(int(n), int(ncube), _ip(csl), _ip(adj_number),
                                _fws_inplace(FWS)) != 0:
        raise BcmgError(f"bcmg_fws_interface: {_lib.last_error()}")


def fws_band_pack(n, FWS, bands):
    """Flag bands (rows of 4 ints: cube slot, axis, side, layers) of FWS
    packed into one int32 buffer, in the state halo's cell order."""
    bands = np.ascontiguousarray(bands, np.int32).reshape(-1, 4)
    total = int(bands[:, 3].sum()) * n * n
    buf = np.zeros(max(total, 1), np.int32)
    F = np.ascontiguousarray(FWS, np.int32)
    if lib().bcmg_fws_band_pack(int(n), F.shape[0], F, len(bands), _ip(bands.reshape(-1)),
                                buf) != 0:
        raise BcmgError(f"bcmg_fws_band_pack: {_lib.last_error()}")
    return buf[:total]


def fws_band_unpack(n, FWS, bands, buf):
    """Writes packed flag bands (fws_band_pack's layout) into FWS in place."""
    bands = np.ascontiguousarray(bands, np.int32).reshape(-1, 4)
    if lib().bcmg_fws_band_unpack(int(n), FWS.shape[0], _fws_inplace(FWS), len(bands),
                                  _ip(bands.reshape(-1)), _ip(buf)) != 0:
        raise BcmgError(f"bcmg_fws_band_unpack: {_lib.last_error()}")


# ---------------------------------------------------------------------------
# Device-resident context
# ---------------------------------------------------------------------------
def _case_desc(case, precision, keep):
    """bcmg_case_desc of one case; the arrays it points at are appended to
    `keep` (they must outlive the create call)."""
    ph = case.phys

    def arr(a, dt):
        a = np.ascontiguousarray(a, dtype=dt)
        if a.size == 0:
            a = np.zeros(1, dt)
        keep.append(a)
        return a.ctypes.data

    xl, xu, yl, yu, zl, zu = case.bc_lists()
    d = _lib.CaseDesc()
    d.n, d.ncube, d.mpi_ncube = case.n, case.ncube, ph.mpi_ncube
    d.mu_L, d.rho0, d.U0, d.Uin, d.P0 = ph.mu_L, ph.rho0, ph.U0, ph.Uin, ph.P0
    d.deltaT, d.deltaTau, d.e = case.dT, case.dTau, case.e
    d.precision = precision
    d.cube_size = arr(case.cube_size, np.float64)
    d.csl = arr(case.csl, np.int32)
    d.adj_number = arr(case.adj, np.int32)
    d.FWS = arr(case.fws, np.int32)
    d.nxl, d.nxu, d.nyl, d.nyu, d.nzl, d.nzu = map(len, (xl, xu, yl, yu, zl, zu))
    d.xl, d.xu, d.yl, d.yu, d.zl, d.zu = (arr(a, np.int32) for a in (xl, xu, yl, yu, zl, zu))
    if case.ibm_minus is not None:
        W, G, I = case.ibm_minus
        d.nminus = (len(G) - 1) // 4
        d.w_minus, d.gc_minus, d.ip_minus = arr(W, np.float64), arr(G, np.int32), arr(I, np.int32)
    if case.ibm_plus is not None:
        W, G, I = case.ibm_plus
        d.nplus = (len(G) - 1) // 4
        d.w_plus, d.gc_plus, d.ip_plus = arr(W, np.float64), arr(G, np.int32), arr(I, np.int32)
    return d


class CaseContext:
    """A case resident in HBM (``bcmg_case_*``)."""

    def __init__(self, case, precision=PRECISION_FP64, nproxy=0):
        """nproxy > 0: a rank's share of a cube-sharded run whose last nproxy
        cube slots are proxies of remote cubes (bcmg_case_create_shard)."""
        self.case = case
        keep = []
        d = _case_desc(case, precision, keep)
        h = C.c_void_p()
        if nproxy:
            check(lib().bcmg_case_create_shard(C.byref(d), int(nproxy), C.byref(h)))
        else:
            check(lib().bcmg_case_create(C.byref(d), C.byref(h)))
        del keep
        self.h = h
        self.shape = case.U.shape
        self.ncase = 1
        self.emax = np.zeros(6)

    def close(self):
        if getattr(self, "h", None):
            lib().bcmg_case_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, U1_=None, U1=None, U1q=None):
        ptr = lambda a: None if a is None else _dp(np.ascontiguousarray(a)).ctypes.data
        keep = [a for a in (U1_, U1, U1q)]
        check(lib().bcmg_case_set_state(self.h, ptr(U1_), ptr(U1), ptr(U1q)))
        del keep

    def get_state(self, out=None):
        """(U1_, U1, U1q) copied to host; `out` may supply the three arrays
        (e.g. pinned buffers)."""
        if out is None:
            out = [np.empty(self.shape) for _ in range(3)]
        for a in out:
            _dp(a)
            if a.shape != tuple(self.shape):
                raise BcmgError("output array has the wrong shape")
        check(lib().bcmg_case_get_state(self.h, *(a.ctypes.data for a in out)))
        return out

    def get_result(self, out=None):
        """The state U1_ alone copied to host (the result of an advance);
        `out` may supply the array (e.g. a pinned buffer)."""
        if out is None:
            out = np.empty(self.shape)
        _dp(out)
        if out.shape != tuple(self.shape):
            raise BcmgError("output array has the wrong shape")
        check(lib().bcmg_case_get_state(self.h, out.ctypes.data, None, None))
        return out

    def get_scratch(self):
        out = [np.empty(self.shape) for _ in range(4)]
        check(lib().bcmg_case_get_scratch(self.h, *(a.ctypes.data for a in out)))
        return out  # U1p1, U1p2, Rku1, Residual1

    def set_method(self, method, cfl=0.0, omega=1.5):
        """Sub-iteration method of advance(): METHOD_RK3 or METHOD_LUSGS
        (pseudo-time CFL, 0 for none; relaxation omega in [1, 4])."""
        check(lib().bcmg_case_set_method(self.h, int(method), float(cfl), float(omega)))

    def stage(self, RK):
        check(lib().bcmg_case_stage(self.h, int(RK)))

    def advance(self, steps, subiters, use_graph=True):
        """er (8 doubles, 1-based like the reference); for a batch [ncase, 8]."""
        er = np.zeros(8 * self.ncase)
        check(lib().bcmg_case_advance(self.h, int(steps), int(subiters), int(bool(use_graph)),
                                      er.ctypes.data, self.emax.ctypes.data))
        return er.reshape(self.ncase, 8) if isinstance(self, BatchContext) else er

    def advance_async(self, steps, subiters):
        """Enqueues `steps` graph-replayed dual-time steps and returns at once
        (bcmg_case_advance_async); norms stay on the device (get_norms)."""
        check(lib().bcmg_case_advance_async(self.h, int(steps), int(subiters)))

    def copy_state_async(self, to_device, U1_=None, U1=None, U1q=None):
        """Enqueues host <-> device copies of the given full arrays (page-
        locked host arrays, left untouched until sync(), make it asynchronous)."""
        ptr = lambda a: None if a is None else _dp(a).ctypes.data
        check(lib().bcmg_case_copy_state_async(self.h, 1 if to_device else 0, ptr(U1_), ptr(U1),
                                               ptr(U1q)))

    def get_norms(self):
        """er of the last step (after waiting for the stream)."""
        er = np.zeros(8 * self.ncase)
        check(lib().bcmg_case_get_norms(self.h, er.ctypes.data, self.emax.ctypes.data))
        return er.reshape(self.ncase, 8) if isinstance(self, BatchContext) else er

    def advance_converged(self, steps, max_subiters, tol=0.02, use_graph=True):
        """Steps with the reference's convergence test (main.cpp:1249-1271);
        returns (er, sub-iterations per step [steps] or [steps, ncase])."""
        er = np.zeros(8 * self.ncase)
        its = np.zeros(max(1, steps) * self.ncase, np.int32)
        check(lib().bcmg_case_advance_converged(
            self.h, int(steps), int(max_subiters), float(tol), int(bool(use_graph)),
            its.ctypes.data, er.ctypes.data, self.emax.ctypes.data))
        its = its[:steps * self.ncase]
        if isinstance(self, BatchContext):
            return er.reshape(self.ncase, 8), its.reshape(steps, self.ncase)
        return er, its

    def output_q(self, path, q=-1, ncube_out=0):
        """PLOT3D solution file of the current state (BCM_Output); returns once
        the device snapshot is queued.  output_wait() waits for the file."""
        check(lib().bcmg_case_output_q(self.h, int(q), int(ncube_out), os.fsencode(path)))

    def output_wait(self):
        check(lib().bcmg_case_output_wait(self.h))

    def output_x(self, path, origin, q=-1, ncube_out=0):
        """PLOT3D grid file from the cube corners origin[ncube][3]."""
        o = np.ascontiguousarray(origin, dtype=np.float64)
        check(lib().bcmg_case_output_x(self.h, int(q), int(ncube_out), os.fsencode(path),
                                       o.ctypes.data))

    def set_tuning(self, flux_tile=0, lusgs_threads=0, flux_form=0):
        """Launch shapes: flux tile edge (0, 4 or 8), threads per cube of the
        split LU-SGS sweep (0: the widest plane) and the split flux form on
        8^3 tiles (1 packed face pairs, 2 one face at a time, 0 default)."""
        t = _lib.Tuning(int(flux_tile), int(lusgs_threads), int(flux_form))
        check(lib().bcmg_case_set_tuning(self.h, C.byref(t)))

    def set_face_copies(self, in_flux=True):
        """Split-precision RK stages and LU-SGS sweeps: make the same-level
        face copies inside the updating kernel (True, default) or in the
        interface call after it (False).  Both give the same bits."""
        check(lib().bcmg_case_set_face_copies(self.h, 1 if in_flux else 0))

    def set_mirror_each_stage(self, on=True):
        """Split precision: form the whole FP32 mirror of the state before
        every flux launch (True) instead of once per dual-time step with the
        state-writing kernels keeping it current (False, default).  Both
        give the same bits."""
        check(lib().bcmg_case_set_mirror_each_stage(self.h, 1 if on else 0))

    def set_concurrent_ghosts(self, on=True):
        """Run the IBM ghost fill beside the boundary fill (True, default;
        only where no cube holds both) or after it (False).  Both give the
        same bits."""
        check(lib().bcmg_case_set_concurrent_ghosts(self.h, 1 if on else 0))

    def concurrent_ghosts(self):
        """Whether the ghost fill runs beside the boundary fill."""
        return bool(lib().bcmg_case_concurrent_ghosts(self.h))

    def autotune(self, reps=3):
        """Times the launch-shape candidates on this context's state, applies the
        fastest and returns the choice with the measured milliseconds."""
        t = _lib.Tuning()
        check(lib().bcmg_case_autotune(self.h, int(reps), C.byref(t)))
        return {"flux_tile": t.flux_tile, "lusgs_threads": t.lusgs_threads,
                "flux_form": t.flux_form,
                "flux_ms": {"8_packed": t.flux_ms[0], "8_single": t.flux_ms[1],
                            "4": t.flux_ms[2]},
                "lusgs_ms": {"widest": t.lusgs_ms[0], "half": t.lusgs_ms[1]}}

    def mirror(self):
        """FP32 mirror of the current state (split-precision path)."""
        out = np.empty(self.shape, np.float32)
        check(lib().bcmg_case_mirror(self.h, out.ctypes.data))
        return out

    def mirror_current(self):
        """The FP32 mirror as the kernels keep it during stepping (not
        re-formed; split-precision path)."""
        out = np.empty(self.shape, np.float32)
        check(lib().bcmg_case_mirror_current(self.h, out.ctypes.data))
        return out

    def sync(self):
        check(lib().bcmg_case_sync(self.h))

    def launch_count(self):
        return int(lib().bcmg_case_launch_count(self.h))

    def time_flux(self, reps=5):
        ms = C.c_double()
        check(lib().bcmg_case_time_flux(self.h, int(reps), C.byref(ms)))
        return ms.value

    def set_profiling(self, on=True):
        check(lib().bcmg_case_set_profiling(self.h, int(bool(on))))

    def profile(self):
        ms = C.c_double()
        n = C.c_longlong()
        check(lib().bcmg_case_profile(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def timer_mark(self, slot):
        check(lib().bcmg_case_timer_mark(self.h, int(slot)))

    def timer_elapsed(self, a, b):
        ms = C.c_double()
        check(lib().bcmg_case_timer_elapsed(self.h, int(a), int(b), C.byref(ms)))
        return ms.value


class BatchContext(CaseContext):
    """Several independent cases (same n) advanced together in one context
    (``bcmg_batch_create``): one flat cube list, per-case constants, norms
    and convergence maxima."""

    def __init__(self, case_list, precision=PRECISION_FP64):
        self.cases = list(case_list)
        keep = []
        descs = (_lib.CaseDesc * len(self.cases))(
            *[_case_desc(c, precision, keep) for c in self.cases])
        h = C.c_void_p()
        check(lib().bcmg_batch_create(len(self.cases), descs, C.byref(h)))
        del keep
        self.h = h
        self.case = None
        self.ncase = len(self.cases)
        n = self.cases[0].n
        self.shape = (1 + sum(c.ncube - 1 for c in self.cases), n + 4, n + 4, n + 4, 5)
        self.emax = np.zeros((self.ncase, 6))

    def case_cubes(self, q):
        """(first flat cube, the case's own cube-slot count)."""
        a, b = C.c_int(), C.c_int()
        check(lib().bcmg_case_case_cubes(self.h, int(q), C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_case_state(self, q, U1_=None, U1=None, U1q=None):
        arrs = [None if a is None else _dp(np.ascontiguousarray(a)) for a in (U1_, U1, U1q)]
        check(lib().bcmg_case_set_case_state(self.h, int(q),
                                             *(None if a is None else a.ctypes.data for a in arrs)))

    def get_case_state(self, q):
        shape = self.cases[q].U.shape
        out = [np.empty(shape) for _ in range(3)]
        check(lib().bcmg_case_get_case_state(self.h, int(q), *(a.ctypes.data for a in out)))
        return out


def probe_fp64_gflops():
    """Measured FP64 FMA rate of the current GPU (GFLOP/s)."""
    g = C.c_double()
    check(lib().bcmg_probe_fp64_rate(C.byref(g)))
    return g.value


# ---------------------------------------------------------------------------
# Cube-sharded runs
# ---------------------------------------------------------------------------
XCHG_HALO = 0
XCHG_NORMS = 1


class ShardedRun:
    """One case split over ranks by cube (the reference's rank_map,
    main.cpp:576-596), run in this process on the current GPU: a context per
    rank (its own cubes, then proxies of the remote cubes its face tasks
    read), each stepped by its own host thread.  The exchange hook of each
    context packs its face bands for every peer into a device buffer, meets
    the other ranks at a host barrier, unpacks the peers' bands into its
    proxies, and for the norms adds the ranks' raw sums in rank order (the
    reference's MPI_Allreduce, BCM_Flux_XYZ_Viscous_Runge_kutta.cpp:2641-2652).
    Ranks meet only at host barriers, so no kernel of one rank ever waits on
    another rank's.  The cells evolve bit for bit as in one context; ranks on
    separate GPUs would move the same buffers with their own transport."""

    def __init__(self, case, rank_of_cube, precision=PRECISION_FP64):
        import threading

        import torch
        self.case = case
        rk = np.asarray(rank_of_cube, np.int32)
        self.nrank = int(rk[1:].max()) + 1
        self.parts = [cases.shard_case(case, rk, r) for r in range(self.nrank)]
        self.ctx = [CaseContext(sub, precision, nproxy=len(prox)) for sub, _, prox in self.parts]
        self._keep = []
        for r, (sub, own, prox) in enumerate(self.parts):
            g2l = np.zeros(case.ncube, np.int32)
            g2l[own] = np.arange(1, len(own) + 1)
            g2l[prox] = np.arange(len(own) + 1, len(own) + len(prox) + 1)
            send, recv = [], []
            for p in range(self.nrank):
                sb = cases.shard_bands(case, rk, r, p) if p != r else np.zeros((0, 4), np.int32)
                rb = cases.shard_bands(case, rk, p, r) if p != r else np.zeros((0, 4), np.int32)
                sb, rb = sb.copy(), rb.copy()
                sb[:, 0] = g2l[sb[:, 0]]
                rb[:, 0] = g2l[rb[:, 0]]
                send.append(np.ascontiguousarray(sb, np.int32))
                recv.append(np.ascontiguousarray(rb, np.int32))
            self._keep += send + recv
            ns = (C.c_int * self.nrank)(*[len(x) for x in send])
            nr = (C.c_int * self.nrank)(*[len(x) for x in recv])
            ps = (C.c_void_p * self.nrank)(*[x.ctypes.data for x in send])
            pr = (C.c_void_p * self.nrank)(*[x.ctypes.data for x in recv])
            check(lib().bcmg_case_set_halo(self.ctx[r].h, self.nrank, ns, ps, nr, pr))
        self.buf = [[None] * self.nrank for _ in range(self.nrank)]
        for r in range(self.nrank):
            for p in range(self.nrank):
                sb, _ = self.halo_bytes(r, p)
                self.buf[r][p] = torch.empty(max(sb, 16), dtype=torch.uint8, device="cuda")
        self.barrier = threading.Barrier(self.nrank)
        self.sums = np.zeros((self.nrank, 7))
        self.error = None
        self._hooks = [_lib.EXCHANGE_FN(self._make_hook(r)) for r in range(self.nrank)]
        for r in range(self.nrank):
            check(lib().bcmg_case_set_exchange(self.ctx[r].h, self._hooks[r], None))

    def halo_bytes(self, r, p):
        a, b = C.c_size_t(), C.c_size_t()
        check(lib().bcmg_case_halo_bytes(self.ctx[r].h, int(p), C.byref(a), C.byref(b)))
        return a.value, b.value

    def _make_hook(self, r):
        L = lib()

        def hook(user, phase, stream):
            try:
                h = self.ctx[r].h
                if phase == XCHG_HALO:
                    for p in range(self.nrank):
                        if p != r:
                            check(L.bcmg_case_halo_pack(h, p, self.buf[r][p].data_ptr()))
                    check(L.bcmg_case_sync(h))
                    self.barrier.wait()  # every rank's bands are packed
                    for p in range(self.nrank):
                        if p != r:
                            check(L.bcmg_case_halo_unpack(h, p, self.buf[p][r].data_ptr()))
                    check(L.bcmg_case_sync(h))
                    self.barrier.wait()  # the buffers may be packed again
                else:
                    s = np.zeros(7)
                    check(L.bcmg_case_norm_sums_host(h, s.ctypes.data, 0))
                    self.sums[r] = s
                    self.barrier.wait()
                    tot = self.sums[0].copy()
                    for p in range(1, self.nrank):  # rank order: the same bits on every rank
                        tot = tot + self.sums[p]
                    check(L.bcmg_case_norm_sums_host(h, tot.ctypes.data, 1))
                    self.barrier.wait()
                return 0
            except Exception as exc:  # reported by the stepping call
                self.error = exc
                self.barrier.abort()
                return 1
        return hook

    def _run(self, fn):
        import threading
        out = [None] * self.nrank
        errs = []

        def work(r):
            try:
                out[r] = fn(self.ctx[r])
            except Exception as exc:
                errs.append(exc)
                self.barrier.abort()

        ts = [threading.Thread(target=work, args=(r,)) for r in range(self.nrank)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()
        if errs or self.error:
            raise BcmgError(f"sharded step failed: {self.error or errs[0]}")
        return out

    def set_state(self, U1_, U1, U1q):
        for (sub, own, prox), ctx in zip(self.parts, self.ctx):
            sl = np.concatenate([[0], own, prox])
            ctx.set_state(U1_[sl], U1[sl], U1q[sl])

    def advance(self, steps, subiters):
        """Dual-time steps on every rank together; returns er (the same on
        every rank)."""
        ers = self._run(lambda c: c.advance(steps, subiters, use_graph=False))
        return ers[0]

    def get_state(self):
        """(U1_, U1, U1q) in the global layout, each cube from its owner."""
        out = [np.array(self.case.U) for _ in range(3)]
        for (sub, own, prox), ctx in zip(self.parts, self.ctx):
            st = ctx.get_state()
            for g, a in zip(out, st):
                g[own] = a[1:1 + len(own)]
        return out

    def close(self):
        for c in self.ctx:
            lib().bcmg_case_set_exchange(c.h, _lib.EXCHANGE_FN(), None)
            c.close()


class DistShard:
    """This process's rank of a cube-sharded run over torch.distributed (one
    process per GPU; RANK/WORLD_SIZE as torchrun sets them): its share of the
    case in one context, the face bands and the norm sums exchanged through
    the process group.  Bands are packed on the GPU, staged through pinned
    host memory and sent with point-to-point messages; the norm sums of all
    ranks are gathered and added in rank order, so every rank finalises the
    same norms.  The exchange runs on the host between kernels, so ranks
    never have kernels waiting on each other (several ranks may share a GPU).
    Works with any backend that moves CPU tensors (gloo)."""

    def __init__(self, case, rank_of_cube, precision=PRECISION_FP64, group=None):
        import torch
        import torch.distributed as dist
        self.dist, self.torch, self.group = dist, torch, group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        rk = np.asarray(rank_of_cube, np.int32)
        if int(rk[1:].max()) + 1 != self.world:
            raise ValueError("rank_of_cube must name every rank of the group")
        self.case = case
        sub, own, prox = cases.shard_case(case, rk, self.rank)
        self.sub, self.own, self.prox = sub, own, prox
        self.ctx = CaseContext(sub, precision, nproxy=len(prox))
        g2l = np.zeros(case.ncube, np.int32)
        g2l[own] = np.arange(1, len(own) + 1)
        g2l[prox] = np.arange(len(own) + 1, len(own) + len(prox) + 1)
        send, recv = [], []
        for p in range(self.world):
            sb = cases.shard_bands(case, rk, self.rank, p) if p != self.rank else np.zeros((0, 4))
            rb = cases.shard_bands(case, rk, p, self.rank) if p != self.rank else np.zeros((0, 4))
            sb, rb = np.array(sb, np.int32), np.array(rb, np.int32)
            sb[:, 0] = g2l[sb[:, 0]]
            rb[:, 0] = g2l[rb[:, 0]]
            send.append(np.ascontiguousarray(sb))
            recv.append(np.ascontiguousarray(rb))
        self._keep = send + recv
        W = self.world
        check(lib().bcmg_case_set_halo(
            self.ctx.h, W, (C.c_int * W)(*[len(x) for x in send]),
            (C.c_void_p * W)(*[x.ctypes.data for x in send]),
            (C.c_int * W)(*[len(x) for x in recv]),
            (C.c_void_p * W)(*[x.ctypes.data for x in recv])))
        self.peers = [p for p in range(W) if p != self.rank]
        self.dbuf, self.hsend, self.hrecv = {}, {}, {}
        for p in self.peers:
            a, b = C.c_size_t(), C.c_size_t()
            check(lib().bcmg_case_halo_bytes(self.ctx.h, p, C.byref(a), C.byref(b)))
            self.dbuf[p] = (torch.empty(max(a.value, 16), dtype=torch.uint8, device="cuda"),
                            torch.empty(max(b.value, 16), dtype=torch.uint8, device="cuda"))
            self.hsend[p] = torch.empty(a.value, dtype=torch.uint8).pin_memory()
            self.hrecv[p] = torch.empty(b.value, dtype=torch.uint8).pin_memory()
        self.error = None
        self._hook = _lib.EXCHANGE_FN(self._exchange)
        check(lib().bcmg_case_set_exchange(self.ctx.h, self._hook, None))

    def _exchange(self, user, phase, stream):
        try:
            L, h, torch, dist = lib(), self.ctx.h, self.torch, self.dist
            if phase == XCHG_HALO:
                for p in self.peers:
                    check(L.bcmg_case_halo_pack(h, p, self.dbuf[p][0].data_ptr()))
                check(L.bcmg_case_sync(h))
                for p in self.peers:
                    self.hsend[p].copy_(self.dbuf[p][0][:self.hsend[p].numel()])
                # a peer's send list is the other's receive list, so both
                # skip the same empty messages
                ops = [dist.P2POp(dist.isend, self.hsend[p], p, self.group)
                       for p in self.peers if self.hsend[p].numel()]
                ops += [dist.P2POp(dist.irecv, self.hrecv[p], p, self.group)
                        for p in self.peers if self.hrecv[p].numel()]
                for w in (dist.batch_isend_irecv(ops) if ops else []):
                    w.wait()
                for p in self.peers:
                    self.dbuf[p][1][:self.hrecv[p].numel()].copy_(self.hrecv[p])
                torch.cuda.synchronize()
                for p in self.peers:
                    check(L.bcmg_case_halo_unpack(h, p, self.dbuf[p][1].data_ptr()))
            else:
                s = np.zeros(7)
                check(L.bcmg_case_norm_sums_host(h, s.ctypes.data, 0))
                got = [torch.zeros(7, dtype=torch.float64) for _ in range(self.world)]
                dist.all_gather(got, torch.from_numpy(s), group=self.group)
                tot = got[0].numpy().copy()
                for p in range(1, self.world):  # rank order: the same bits everywhere
                    tot = tot + got[p].numpy()
                check(L.bcmg_case_norm_sums_host(h, tot.ctypes.data, 1))
            return 0
        except Exception as exc:
            self.error = exc
            return 1

    def set_state(self, U1_, U1, U1q):
        sl = np.concatenate([[0], self.own, self.prox])
        self.ctx.set_state(U1_[sl], U1[sl], U1q[sl])

    def advance(self, steps, subiters):
        try:
            return self.ctx.advance(steps, subiters, use_graph=False)
        except BcmgError:
            if self.error:
                raise BcmgError(f"sharded step failed: {self.error}")
            raise

    def own_state(self):
        """(own cubes, U1_, U1, U1q of those cubes)."""
        st = self.ctx.get_state()
        k = len(self.own)
        return self.own, st[0][1:1 + k], st[1][1:1 + k], st[2][1:1 + k]

    def close(self):
        lib().bcmg_case_set_exchange(self.ctx.h, _lib.EXCHANGE_FN(), None)
        self.ctx.close()
