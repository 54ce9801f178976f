"""ORACLE (test infrastructure): Python access to the CPU checkers.

* ``Port`` wraps ``oracle/bcm_oracle.c`` (the C restatement, any resolution),
  built by ``build_port()`` with ``gcc -O2 -ffp-contract=off`` into
  ``oracle/_build/``.
* ``Ref`` wraps the reference's own compiled sources (``oracle/ref_build.py``),
  one library per compile-time configuration; available only where the
  reference sources are present.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use
this module, and only as the checker / the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
sys.path.insert(0, HERE)
import ref_build  # noqa: E402

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def build_port(force: bool = False) -> str:
    """Compile the C restatement; returns the .so path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    out = os.path.join(BUILD_DIR, "libbcm_oracle.so")
    srcs = [os.path.join(HERE, "bcm_oracle.c"), os.path.join(HERE, "bcm_oracle_lusgs.c"),
            os.path.join(HERE, "bcm_oracle_ibm.c")]
    hdr = os.path.join(HERE, "bcm_oracle.h")
    if (not force and os.path.isfile(out) and os.path.getmtime(out) >= max(
            [os.path.getmtime(x) for x in srcs] + [os.path.getmtime(hdr)])):
        return out
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-std=c11",
           *srcs, "-o", out + ".tmp", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stderr[-4000:])
    os.replace(out + ".tmp", out)
    return out


class _PhysC(C.Structure):
    _fields_ = [("n", C.c_int), ("mpi_ncube", C.c_int), ("mu_L", C.c_double),
                ("rho0", C.c_double), ("U0", C.c_double), ("Uin", C.c_double),
                ("P0", C.c_double)]


def _ibm(case, which):
    t = case.ibm_minus if which < 0 else case.ibm_plus
    if t is None:
        return 0, np.zeros(9), np.zeros(5, np.int32), np.zeros(5, np.int32)
    W, G, I = t
    return (len(G) - 1) // 4, np.ascontiguousarray(W, np.float64), \
        np.ascontiguousarray(G, np.int32), np.ascontiguousarray(I, np.int32)


class State:
    """The mutable arrays of one run (reference layout)."""

    def __init__(self, case):
        self.U1_ = np.ascontiguousarray(case.U.copy())
        self.U1 = self.U1_.copy()
        self.U1q = self.U1_.copy()
        self.U1p1 = np.zeros_like(self.U1_)
        self.U1p2 = np.zeros_like(self.U1_)
        self.Rku1 = np.zeros_like(self.U1_)
        # Residual1 is zeroed explicitly: the reference allocates it with
        # new[] and sums all interior cells (BCM_Flux...cpp:2609-2610).
        self.Residual1 = np.zeros_like(self.U1_)
        self.er = np.zeros(8)
        self.Emax = np.zeros(6)

    def arrays(self):
        return dict(U1_=self.U1_, U1=self.U1, U1q=self.U1q, U1p1=self.U1p1, U1p2=self.U1p2,
                    Rku1=self.Rku1, Residual1=self.Residual1, er=self.er)


class Port:
    """The C restatement."""

    def __init__(self):
        self.lib = C.CDLL(build_port())
        L = self.lib
        P = C.POINTER(_PhysC)
        L.bcmo_flux_stage.argtypes = [P, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                      _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.bcmo_bc.argtypes = [P, C.c_int, C.c_int, _ip, _ip, C.c_int, C.c_int, _ip, _ip,
                              C.c_int, C.c_int, _ip, _ip, _dp]
        L.bcmo_ghost.argtypes = [P, C.c_int, _dp, _ip, _ip, _dp]
        L.bcmo_interface.argtypes = [P, C.c_int, _ip, _ip, _dp]
        L.bcmo_time_shift.argtypes = [P, C.c_int, _dp, _dp, _dp]
        L.bcmo_run.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                               C.c_double, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                               _dp, C.c_int, C.c_int, _ip, _ip, C.c_int, C.c_int, _ip, _ip,
                               C.c_int, C.c_int, _ip, _ip, C.c_int, _dp, _ip, _ip, C.c_int,
                               _dp, _ip, _ip, _dp, _dp]
        L.bcmo_run_lusgs.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                     C.c_double, C.c_double, _ip, _ip, _ip, _dp, _dp, _dp,
                                     _dp, _dp, _dp, C.c_int, C.c_int, _ip, _ip, C.c_int,
                                     C.c_int, _ip, _ip, C.c_int, C.c_int, _ip, _ip, C.c_int,
                                     _dp, _ip, _ip, C.c_int, _dp, _ip, _ip, _dp, _dp]
        L.bcmo_lusgs.argtypes = [P, C.c_int, C.c_double, C.c_double, C.c_double, _ip, _dp,
                                 _dp, _dp, _dp, _dp]
        L.bcmo_run_converged.argtypes = [P, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                         C.c_double, C.c_double, C.c_double, C.c_double,
                                         C.c_double, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp,
                                         _dp, _dp, C.c_int, C.c_int, _ip, _ip, C.c_int, C.c_int,
                                         _ip, _ip, C.c_int, C.c_int, _ip, _ip, C.c_int, _dp, _ip,
                                         _ip, C.c_int, _dp, _ip, _ip, _dp, _dp, _ip]
        L.bcmo_ibm.argtypes = [C.c_int, C.c_int, _dp, _ip, _dp, _dp, _dp, _ip, C.c_int, _dp,
                               C.c_int, C.POINTER(C.c_int), _ip, _ip, _dp, C.POINTER(C.c_int),
                               _ip, _ip, _dp, _dp]
        L.bcmo_set_threads.argtypes = [C.c_int]

    @staticmethod
    def phys(case):
        ph = case.phys
        return C.byref(_PhysC(case.n, ph.mpi_ncube, ph.mu_L, ph.rho0, ph.U0, ph.Uin, ph.P0))

    def set_threads(self, n):
        self.lib.bcmo_set_threads(int(n))

    def flux_stage(self, case, st: State, RK: int):
        self.lib.bcmo_flux_stage(self.phys(case), case.ncube, RK, case.dT, case.dTau, case.e,
                                 case.fws, case.cube_size, st.U1_, st.U1, st.U1q, st.U1p1,
                                 st.U1p2, st.Rku1, st.Residual1, st.er)

    def bc(self, case, U):
        xl, xu, yl, yu, zl, zu = case.bc_lists()
        self.lib.bcmo_bc(self.phys(case), len(xl), len(xu), _nz(xl), _nz(xu), len(yl),
                         len(yu), _nz(yl), _nz(yu), len(zl), len(zu), _nz(zl), _nz(zu), U)

    def ghost(self, case, U, which):
        nb, W, G, I = _ibm(case, which)
        if nb:
            self.lib.bcmo_ghost(self.phys(case), nb, W, G, I, U)

    def interface(self, case, U):
        self.lib.bcmo_interface(self.phys(case), case.ncube, _adj(case), case.csl, U)

    def time_shift(self, case, st: State):
        self.lib.bcmo_time_shift(self.phys(case), case.ncube, st.U1_, st.U1, st.U1q)

    def run_lusgs(self, case, st: State, steps: int, subiters: int, cfl: float = 0.0,
                  omega: float = 1.5):
        """bcmo_run with one LU-SGS update per sub-iteration (no reference
        counterpart; see bcm_oracle_lusgs.c)."""
        xl, xu, yl, yu, zl, zu = case.bc_lists()
        nm, Wm, Gm, Im = _ibm(case, -1)
        npl, Wp, Gp, Ip = _ibm(case, 1)
        self.lib.bcmo_run_lusgs(self.phys(case), case.ncube, steps, subiters, case.dT, cfl,
                                omega, case.e, case.fws, _adj(case), case.csl, case.cube_size,
                                st.U1_, st.U1, st.U1q, st.Rku1, st.Residual1, len(xl), len(xu),
                                _nz(xl), _nz(xu), len(yl), len(yu), _nz(yl), _nz(yu), len(zl),
                                len(zu), _nz(zl), _nz(zu), nm, Wm, Gm, Im, npl, Wp, Gp, Ip,
                                st.er, st.Emax)

    def run_converged(self, case, st: State, steps: int, max_subiters: int, tol: float,
                      method: int = 0, cfl: float = 0.0, omega: float = 1.5):
        """The reference loop with its convergence test (main.cpp:1249-1271);
        returns the sub-iteration count of each step."""
        xl, xu, yl, yu, zl, zu = case.bc_lists()
        nm, Wm, Gm, Im = _ibm(case, -1)
        npl, Wp, Gp, Ip = _ibm(case, 1)
        iters = np.zeros(max(1, steps), np.int32)
        self.lib.bcmo_run_converged(
            self.phys(case), case.ncube, steps, max_subiters, tol, method, case.dT, case.dTau,
            cfl, omega, case.e, case.fws, _adj(case), case.csl, case.cube_size, st.U1_, st.U1,
            st.U1q, st.U1p1, st.U1p2, st.Rku1, st.Residual1, len(xl), len(xu), _nz(xl), _nz(xu),
            len(yl), len(yu), _nz(yl), _nz(yu), len(zl), len(zu), _nz(zl), _nz(zu), nm, Wm, Gm,
            Im, npl, Wp, Gp, Ip, st.er, st.Emax, iters)
        return iters[:steps]

    def ibm(self, case, fws, tris):
        """IBM preprocessing (restatement of BCM_Immersed_boundary) for the
        triangles tris[ntri, 3, 3]; fws updated in place.  Returns the minus
        and plus tables as (GCindex[m,4], IPsur[m,4], weight[m,8])."""
        tri = np.ascontiguousarray(np.asarray(tris, np.float64).reshape(-1, 9))
        ntri = tri.shape[0]
        cap = int((fws == 0).sum()) + 1
        o = np.ascontiguousarray(case.origin, dtype=np.float64)
        out = [np.zeros(4 * cap, np.int32), np.zeros(4 * cap, np.int32), np.zeros(8 * cap),
               np.zeros(4 * cap, np.int32), np.zeros(4 * cap, np.int32), np.zeros(8 * cap)]
        nm, npl = C.c_int(), C.c_int()
        r = self.lib.bcmo_ibm(case.n, case.ncube, np.ascontiguousarray(case.cube_size, np.float64),
                              np.ascontiguousarray(case.csl, np.int32),
                              np.ascontiguousarray(o[:, 0]), np.ascontiguousarray(o[:, 1]),
                              np.ascontiguousarray(o[:, 2]), fws, ntri,
                              tri if ntri else np.zeros(9), cap, C.byref(nm), out[0], out[1],
                              out[2], C.byref(npl), out[3], out[4], out[5],
                              np.zeros(max(9 * ntri, 9)))
        if r != 0:
            raise RuntimeError("bcmo_ibm: table capacity exceeded")
        m, p = nm.value, npl.value
        return ((out[0][:4 * m].reshape(m, 4), out[1][:4 * m].reshape(m, 4),
                 out[2][:8 * m].reshape(m, 8)),
                (out[3][:4 * p].reshape(p, 4), out[4][:4 * p].reshape(p, 4),
                 out[5][:8 * p].reshape(p, 8)))

    def residual(self, case, st: State):
        """The raw residual R(U1_) into st.Rku1 (fluid cells) and the force
        integrands into st.Residual1 (bcmo_flux_stage with RK = 0)."""
        self.flux_stage(case, st, 0)

    def run(self, case, st: State, steps: int, subiters: int):
        xl, xu, yl, yu, zl, zu = case.bc_lists()
        nm, Wm, Gm, Im = _ibm(case, -1)
        npl, Wp, Gp, Ip = _ibm(case, 1)
        self.lib.bcmo_run(self.phys(case), case.ncube, steps, subiters, case.dT, case.dTau,
                          case.e, case.fws, _adj(case), case.csl, case.cube_size, st.U1_,
                          st.U1, st.U1q, st.U1p1, st.U1p2, st.Rku1, st.Residual1, len(xl),
                          len(xu), _nz(xl), _nz(xu), len(yl), len(yu), _nz(yl), _nz(yu),
                          len(zl), len(zu), _nz(zl), _nz(zu), nm, Wm, Gm, Im, npl, Wp, Gp, Ip,
                          st.er, st.Emax)


def _nz(a):
    """Non-empty int32 array (a zero-length list still needs a valid pointer)."""
    a = np.ascontiguousarray(a, np.int32)
    return a if a.size else np.zeros(1, np.int32)


def _one_based(a):
    """Reference lists are 1-based: element 0 unused."""
    return np.concatenate([np.zeros(1, np.int32), np.ascontiguousarray(a, np.int32)])


def _adj(case):
    return np.ascontiguousarray(case.adj, np.int32)


def ref_config_for(case) -> "ref_build.RefConfig":
    ph = case.phys
    tag = f"n{case.n}_m{ph.mpi_ncube}_{abs(hash((ph.mu_L, ph.rho0, ph.U0, ph.Uin, ph.P0))) % 10**8}"
    return ref_build.RefConfig(tag, ncube_x=case.n, mpi_ncube=ph.mpi_ncube, mu_L=ph.mu_L,
                               rho0=ph.rho0, U0=ph.U0, Uin=ph.Uin, P0=ph.P0)


class Ref:
    """The reference's own compiled sources for the case's compile-time config."""

    def __init__(self, case):
        path = ref_build.build(ref_config_for(case))
        if path is None:
            raise FileNotFoundError("reference sources not available on this machine")
        self.lib = C.CDLL(path)
        L = self.lib
        L.ref_flux.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _ip, _ip,
                               _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.ref_bc.argtypes = [C.c_int, C.c_int, _ip, _ip, C.c_int, C.c_int, _ip, _ip, C.c_int,
                             C.c_int, _ip, _ip, _dp]
        L.ref_ghost.argtypes = [C.c_int, C.c_int, _dp, _ip, _ip, _ip, _dp]
        L.ref_interface_setup.argtypes = [C.c_int, _ip, _ip, _ip]
        L.ref_interface.argtypes = [_dp]
        L.ref_interface_list.argtypes = [C.c_int, _ip]
        L.ref_set_threads.argtypes = [C.c_int]
        L.ref_output.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.ref_ibm.argtypes = [C.c_int, _dp, _ip, _dp, _dp, _dp, _ip]
        L.ref_fws_interface.argtypes = [_ip]
        L.ref_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                              _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int,
                              C.c_int, _ip, _ip, C.c_int, C.c_int, _ip, _ip, C.c_int, C.c_int,
                              _ip, _ip, C.c_int, _dp, _ip, _ip, C.c_int, _dp, _ip, _ip, _dp,
                              _dp]
        assert L.ref_ncube_x() == case.n
        self.counts = np.zeros(15, np.int32)
        L.ref_interface_setup(case.ncube, _adj(case), case.csl, self.counts)
        self.case = case

    def set_threads(self, n):
        self.lib.ref_set_threads(int(n))

    def flux_stage(self, case, st: State, RK: int):
        self.lib.ref_flux(case.ncube, RK, case.dT, case.dTau, case.e, case.fws, case.csl,
                          case.cube_size, st.U1_, st.U1, st.U1q, st.U1p1, st.U1p2, st.Rku1,
                          st.Residual1, st.er)

    def bc(self, case, U):
        xl, xu, yl, yu, zl, zu = (_one_based(a) for a in case.bc_lists())
        self.lib.ref_bc(len(xl) - 1, len(xu) - 1, xl, xu, len(yl) - 1, len(yu) - 1, yl, yu,
                        len(zl) - 1, len(zu) - 1, zl, zu, U)

    def ghost(self, case, U, which):
        nb, W, G, I = _ibm(case, which)
        if nb:
            self.lib.ref_ghost(which, nb, W, G, I, case.fws, U)

    def interface(self, case, U):
        self.lib.ref_interface(U)

    def output(self, case, U, step: int, directory: str):
        """The reference's BCM_Output of U into `directory` (BCMdata00001.x and
        qBCMdata<step>.q)."""
        cwd = os.getcwd()
        os.chdir(directory)
        try:
            o = np.ascontiguousarray(case.origin, dtype=np.float64)
            self.lib.ref_output(case.ncube, step, U, case.cube_size,
                                np.ascontiguousarray(o[:, 0]), np.ascontiguousarray(o[:, 1]),
                                np.ascontiguousarray(o[:, 2]))
        finally:
            os.chdir(cwd)

    def ibm(self, case, fws, directory: str):
        """The reference's BCM_Immersed_boundary in `directory` (which holds
        BCM_STL_fine.stl); fws (the case's flags) is updated in place."""
        cwd = os.getcwd()
        os.chdir(directory)
        try:
            o = np.ascontiguousarray(case.origin, dtype=np.float64)
            self.lib.ref_ibm(case.ncube, np.ascontiguousarray(case.cube_size, dtype=np.float64),
                             np.ascontiguousarray(case.csl, dtype=np.int32),
                             np.ascontiguousarray(o[:, 0]), np.ascontiguousarray(o[:, 1]),
                             np.ascontiguousarray(o[:, 2]), fws)
        finally:
            os.chdir(cwd)

    def fws_interface(self, case, fws):
        """The reference's BCM_FWS_Interface on one rank, with the same-level
        lists its BCM_Interface_table built for the case; fws (the case's
        flags, int32 [ncube][n+4]^3) is updated in place."""
        self.lib.ref_fws_interface(fws)

    def run(self, case, st: State, steps: int, subiters: int):
        xl, xu, yl, yu, zl, zu = (_one_based(a) for a in case.bc_lists())
        nm, Wm, Gm, Im = _ibm(case, -1)
        npl, Wp, Gp, Ip = _ibm(case, 1)
        self.lib.ref_run(case.ncube, steps, subiters, case.dT, case.dTau, case.e, case.fws,
                         case.csl, case.cube_size, st.U1_, st.U1, st.U1q, st.U1p1, st.U1p2,
                         st.Rku1, st.Residual1, len(xl) - 1, len(xu) - 1, xl, xu, len(yl) - 1,
                         len(yu) - 1, yl, yu, len(zl) - 1, len(zu) - 1, zl, zu, nm, Wm, Gm, Im,
                         npl, Wp, Gp, Ip, st.er, st.Emax)


def fws_interface(n, ncube, csl, adj, fws):
    """Restatement of BCM_FWS_Interface (BCM_FWS_Interface.cpp:23-791) on one
    rank, in numpy; returns the new flags (int32 [ncube][n+4]^3).

    * A double copy of the flags of every finest-level cube (csl == 0)
      (:111-131); other cubes are never thresholded, so their copy is unused.
    * Same-level pairs: a cube with any of adj[c][1..4][dir] > 0 whose
      largest slot value is a cube of the same level, per axis in cube order
      (BCM_Interface_table.cpp:96-120); the neighbour is adj[c][1][dir].
      The neighbour's low ghost layers take the cube's layers n, n+1 and the
      cube's high ghost layers the neighbour's layers 2, 3, over the face's
      interior (:555-660), X, then Y, then Z.
    * Threshold at +-0.5 back to -1 / 0 / 1 (:668-700).
    * Holes (:702-783): a cell with every index in 1..n+2, flag >= 0, and
      both neighbours along some axis at -1 becomes -1, until none changes.
      The reference sweeps in place in memory order; the rule is monotone,
      so all cells of a Jacobi round change at once here and the fixed point
      is the same.
    """
    S = n + 4
    fws = np.ascontiguousarray(fws, np.int32)
    csl = np.asarray(csl)
    adj = np.asarray(adj).reshape(ncube, 5, 7)
    T = fws.astype(np.float64)
    I = slice(2, n + 2)
    for ax in range(3):
        d = 2 + 2 * ax
        for c in range(1, ncube):
            slots = adj[c, 1:5, d]
            if not (slots > 0).any() or csl[c] != csl[slots.max()]:
                continue
            c2 = adj[c, 1, d]
            for l in range(2):
                lo, src, hi, src2 = [[I, I, I] for _ in range(4)]
                lo[ax], src[ax], hi[ax], src2[ax] = l, n + l, n + 2 + l, 2 + l
                T[(c2, *lo)] = T[(c, *src)]
                T[(c, *hi)] = T[(c2, *src2)]
    out = fws.copy()
    lv = np.nonzero(csl[:ncube] == 0)[0]
    lv = lv[lv >= 1]
    if len(lv):
        t = T[lv]
        F = np.where(t > 0.5, 1, np.where(t < -0.5, -1, 0)).astype(np.int32)
        R = slice(1, n + 3)
        while True:
            core = F[:, R, R, R]
            pair = np.zeros(core.shape, bool)
            for ax in range(3):
                up, dn = [slice(None), R, R, R], [slice(None), R, R, R]
                up[1 + ax] = slice(2, n + 4)
                dn[1 + ax] = slice(0, n + 2)
                pair |= (F[tuple(up)] + F[tuple(dn)]) == -2
            hole = (core >= 0) & pair
            if not hole.any():
                break
            core[hole] = -1
        out[lv] = F
    assert out.shape == (ncube, S, S, S)
    return out


def reference_available() -> bool:
    return ref_build.reference_available()
