"""CPU model of the stage sequence, checking the interface plan the library
builds (bcmg_interface_plan): the reduced opening face-copy list and the
same-level push table leave every cell as the reference's order does.

The model keeps one value per cell and mimics what each kernel writes and
reads: boundary fills on their ghost faces (BCM_X/Y/Z_boundary_condition:
x faces over interior j, k; y faces over all i, interior k; z faces over all
i, j), IBM ghost cells from their 2x2x2 stencils in table order
(BCM_Ghostcell_minus.cpp:72), same-level copies, level-jump injection and
averaging (BCM_Interface.cpp:1745-4358), the three-phase edge fill
(:5640-5732), and an update of fluid interior cells.  The reference runs
boundaries, ghost cells, the full interface, the update and the full
interface again every stage (main.cpp:1161-1207).  The library's order
runs the reduced list ahead of every stage but a step's first, and the
updating kernel copies the same-level faces of the cells it changes, so the
closing call keeps only the level jumps and the edge fill; after RK stages
1 and 2 it keeps only the level jumps and edge fills that the next stage's
boundary fill or IBM stencils read before its opening call rewrites them
(bcmg_interface_closing_plan)."""
import ctypes as C

import numpy as np
import pytest

from bcm_cgli_gb300 import cases
from bcm_cgli_gb300._lib import lib


def _plan(case):
    adj = np.ascontiguousarray(case.adj, np.int32)
    csl = np.ascontiguousarray(case.csl, np.int32)
    cap = 24 * case.ncube
    off = np.zeros(case.ncube + 1, np.int32)
    words = np.zeros(5 * cap, np.int32)
    nt = lib().bcmg_interface_tasks(case.ncube, adj, csl, off, words, cap)
    assert nt >= 0
    lists = [np.ascontiguousarray(a, np.int32) for a in case.bc_lists()]
    ptrs = (C.c_void_p * 6)(*[a.ctypes.data if len(a) else None for a in lists])
    counts = (C.c_int * 6)(*[len(a) for a in lists])
    g = [None if t is None else np.ascontiguousarray(t[1], np.int32)
         for t in (case.ibm_minus, case.ibm_plus)]
    keep = np.zeros(max(nt, 1), np.int32)
    push = np.zeros(6 * case.ncube, np.int32)
    r = lib().bcmg_interface_plan(case.n, case.ncube, adj, csl, C.cast(ptrs, C.c_void_p),
                                  C.cast(counts, C.c_void_p),
                                  None if g[0] is None else g[0].ctypes.data,
                                  0 if g[0] is None else (len(g[0]) - 1) // 4,
                                  None if g[1] is None else g[1].ctypes.data,
                                  0 if g[1] is None else (len(g[1]) - 1) // 4,
                                  keep, push, cap)
    assert r == nt
    tasks = words[:5 * nt].reshape(-1, 5)
    dst = np.repeat(np.arange(case.ncube), np.diff(off))
    ipt = [None if t is None else np.ascontiguousarray(t[2], np.int32)
           for t in (case.ibm_minus, case.ibm_plus)]
    keep_q = np.zeros(max(nt, 1), np.int32)
    edge = np.zeros(case.ncube, np.int32)
    r = lib().bcmg_interface_closing_plan(case.n, case.ncube, adj, csl, C.cast(ptrs, C.c_void_p),
                                          C.cast(counts, C.c_void_p),
                                          None if ipt[0] is None else ipt[0].ctypes.data,
                                          0 if ipt[0] is None else (len(ipt[0]) - 1) // 4,
                                          None if ipt[1] is None else ipt[1].ctypes.data,
                                          0 if ipt[1] is None else (len(ipt[1]) - 1) // 4,
                                          keep_q, edge, cap)
    assert r == nt
    return (tasks, dst, keep[:nt].astype(bool), push.reshape(case.ncube, 6),
            keep_q[:nt].astype(bool), edge.astype(bool))


class Model:
    def __init__(self, case, seed):
        self.n, self.S, self.case = case.n, case.S, case
        rng = np.random.default_rng(seed)
        self.X = rng.standard_normal((case.ncube, case.S, case.S, case.S))
        self.fluid = case.fws == 1
        self.tasks, self.dst, self.keep, self.push, self.keep_q, self.edge_q = _plan(case)
        self.bc = [(c, m) for c, m in self._bc_masks().items()]
        self.ibm = []
        for t in (case.ibm_minus, case.ibm_plus):
            if t is not None:
                G = np.asarray(t[1][1:]).reshape(-1, 4)
                P = np.asarray(t[2][1:]).reshape(-1, 4)
                self.ibm += list(zip(map(tuple, G), map(tuple, P)))

    def _bc_masks(self):
        m = {}
        for bit, lst in enumerate(self.case.bc_lists()):
            for c in lst:
                m[int(c)] = m.get(int(c), 0) | (1 << bit)
        return m

    # -- kernels -----------------------------------------------------------
    def boundary(self):
        n, X = self.n, self.X
        I = slice(2, n + 2)
        for c, m in self.bc:
            Q = X[c]
            if m & 1:
                Q[0:2, I, I] = 1.5 * Q[2, I, I]
            if m & 2:
                Q[n + 2:n + 4, I, I] = Q[n + 1, I, I]
            if m & 4:
                Q[:, 0:2, I] = Q[:, 2:3, I]
            if m & 8:
                Q[:, n + 2:n + 4, I] = Q[:, n + 1:n + 2, I]
            if m & 16:
                Q[:, :, 0:2] = -Q[:, :, 2:3]
            if m & 32:
                Q[:, :, n + 2:n + 4] = Q[:, :, n + 1:n + 2]

    def ghosts(self):
        X = self.X
        for (g, gi, gj, gk), (c, i, j, k) in self.ibm:
            X[g, gi, gj, gk] = 0.9 * X[c, i:i + 2, j:j + 2, k:k + 2].mean()

    def _region(self, ax, layers):
        n = self.n
        sl = [slice(2, n + 2)] * 3
        sl[ax] = slice(layers[0], layers[1] + 1)
        return tuple(sl)

    def _copy(self, t):
        src, ax, side, kind, slot = (int(v) for v in self.tasks[t])
        c, n, X = int(self.dst[t]), self.n, self.X
        h = n // 2
        if kind == 0:
            d = (0, 1) if side == 0 else (n + 2, n + 3)
            s = (n, n + 1) if side == 0 else (2, 3)
            X[(c,) + self._region(ax, d)] = X[(src,) + self._region(ax, s)]
            return
        t0, t1 = (1, 2) if ax == 0 else ((0, 2) if ax == 1 else (0, 1))
        o0 = h if slot in (2, 4) else 0
        o1 = h if slot in (3, 4) else 0
        if kind == 1:  # coarse -> fine injection, both ghost layers alike
            gs = n + 1 if side == 0 else 2
            for l in range(2):
                for p in range(2, n + 2):
                    for q in range(2, n + 2):
                        d, sr = [0] * 3, [0] * 3
                        d[ax], d[t0], d[t1] = (l if side == 0 else n + 2 + l), p, q
                        sr[ax], sr[t0], sr[t1] = gs, p // 2 + 1 + o0, q // 2 + 1 + o1
                        X[(c,) + tuple(d)] = X[(src,) + tuple(sr)]
        else:  # fine -> coarse: 2x2x2 average into the slot's quadrant
            for l in range(2):
                for p in range(2, h + 2):
                    for q in range(2, h + 2):
                        d, b = [0] * 3, [0] * 3
                        d[ax] = n + 2 + l if side == 1 else l
                        d[t0], d[t1] = p + o0, q + o1
                        b[ax] = 2 * (l + 1) if side == 1 else n - 2 + 2 * l
                        b[t0], b[t1] = (p - 1) * 2, (q - 1) * 2
                        X[(c,) + tuple(d)] = X[src, b[0]:b[0] + 2, b[1]:b[1] + 2,
                                               b[2]:b[2] + 2].mean()

    def _edges(self, cubes=None):
        n, X = self.n, self.X
        nx, nyy = n + 1, n + 2
        for c in range(1, self.case.ncube):
            if cubes is not None and not cubes[c]:
                continue
            Q = X[c]
            for i in range(2, nx + 1):
                Q[i, 1, 1] = 0.5 * (Q[i, 1, 2] + Q[i, 2, 1])
                Q[i, nyy, 1] = 0.5 * (Q[i, nyy, 2] + Q[i, nx, 1])
                Q[i, 1, nyy] = 0.5 * (Q[i, 1, nx] + Q[i, 2, nyy])
                Q[i, nyy, nyy] = 0.5 * (Q[i, nyy, nx] + Q[i, nx, nyy])
            for j in range(1, nyy + 1):
                Q[1, j, 1] = 0.5 * (Q[1, j, 2] + Q[2, j, 1])
                Q[1, j, nyy] = 0.5 * (Q[2, j, nyy] + Q[1, j, nx])
                Q[nyy, j, 1] = 0.5 * (Q[nx, j, 1] + Q[nyy, j, 2])
                Q[nyy, j, nyy] = 0.5 * (Q[nx, j, nyy] + Q[nyy, j, nx])
            for k in range(1, nyy + 1):
                Q[1, 1, k] = 0.5 * (Q[1, 2, k] + Q[2, 1, k])
                Q[1, nyy, k] = 0.5 * (Q[2, nyy, k] + Q[1, nx, k])
                Q[nyy, 1, k] = 0.5 * (Q[nx, 1, k] + Q[nyy, 2, k])
                Q[nyy, nyy, k] = 0.5 * (Q[nx, nyy, k] + Q[nyy, nx, k])

    def interface(self, which, edge_cubes=None):
        for t in np.nonzero(which)[0]:
            self._copy(t)
        self._edges(edge_cubes)

    def update(self, stage, push):
        n, X = self.n, self.X
        I = slice(2, n + 2)
        inc = 0.01 * np.sin(stage + X[:, I, I, I])
        X[:, I, I, I] += np.where(self.fluid[:, I, I, I], inc, 0.0)
        if not push:
            return
        for c in range(1, self.case.ncube):
            for ax in range(3):
                for slot, (layers, shift) in enumerate((((2, 3), n), ((n, n + 1), -n))):
                    d = int(self.push[c, 2 * ax + slot])
                    if d <= 0:
                        continue
                    src = self._region(ax, layers)
                    dl = (layers[0] + shift, layers[1] + shift)
                    dst = self._region(ax, dl)
                    X[(d,) + dst] = np.where(self.fluid[(c,) + src], X[(c,) + src], X[(d,) + dst])


def _run(case, library_order, steps=2, subiters=2, push=None, reduced_closing=None,
         ghost_first=False):
    m = Model(case, seed=5)
    push = library_order if push is None else push
    reduced_closing = library_order if reduced_closing is None else reduced_closing
    every = np.ones(len(m.tasks), bool)
    level = m.tasks[:, 3] != 0
    stage = 0
    for _ in range(steps):
        for it in range(subiters):
            for rk in range(3):
                first = it == 0 and rk == 0
                if ghost_first:  # the ghost fill no longer waits for the boundary fill
                    m.ghosts()
                    m.boundary()
                else:
                    m.boundary()
                    m.ghosts()
                m.interface(every if (first or not library_order) else m.keep)
                m.update(stage, push=push)
                if not library_order:
                    m.interface(every)
                elif reduced_closing and rk < 2:  # RK 1, 2: what is read before the next
                    m.interface(m.keep_q, m.edge_q)  # opening call rewrites it
                else:
                    m.interface(level)
                stage += 1
    return m.X


@pytest.mark.parametrize("make", [
    lambda: cases.taylor_green(ncx=3, n=4),
    lambda: cases.random_case(seed=3, n=8, periodic=True),
    lambda: cases.random_case(seed=11, n=4, periodic=False),
    lambda: cases.random_two_level_case(seed=1, n=4),
    lambda: cases.random_two_level_case(seed=6, n=8, periodic=False),
    lambda: cases.sphere_ibm(n=8, coarse=2.0, box=((-2, 4), (-2, 2), (-2, 2)),
                             refine_box=((-2, 2), (-2, 2), (-2, 2))),
    lambda: cases.random_case(seed=24, ncx=1, ncy=1, ncz=1, n=4, periodic=True),
    lambda: cases.random_case(seed=25, ncx=3, ncy=2, ncz=1, n=4, periodic=False)],
    ids=["tgv_periodic", "random_periodic_ibm", "random_open_ibm", "two_level_periodic",
         "two_level_open", "sphere_two_level_ibm", "one_cube_periodic", "open_3x2x1"])
def test_library_order_equals_reference_order(make):
    case = make()
    a = _run(case, library_order=False)
    b = _run(case, library_order=True)
    assert np.array_equal(a[1:], b[1:])


def test_model_detects_a_missing_copy():
    """The model is sharp: dropping one kept task from the reduced list (a
    face the boundary fill writes), or the in-kernel copies, changes the
    result."""
    case = cases.random_case(seed=11, n=4, periodic=False)
    m = Model(case, seed=5)
    kept_same = np.nonzero(m.keep & (m.tasks[:, 3] == 0))[0]
    assert len(kept_same) > 0
    ref = _run(case, library_order=True)
    orig = Model.__init__

    def patched(self, case, seed):
        orig(self, case, seed)
        self.keep = self.keep.copy()
        self.keep[kept_same[0]] = False
    Model.__init__ = patched
    try:
        bad = _run(case, library_order=True)
    finally:
        Model.__init__ = orig
    assert not np.array_equal(ref[1:], bad[1:])
    # and the closing call without the in-kernel copies loses them
    assert not np.array_equal(ref[1:], _run(case, library_order=True, push=False)[1:])


@pytest.mark.parametrize("make,drop", [
    (lambda: cases.random_case(seed=11, n=4, periodic=False), "edges"),
    (lambda: cases.random_two_level_case(seed=6, n=8, periodic=False), "tasks")],
    ids=["random_open_ibm_edges", "two_level_open_tasks"])
def test_reduced_closing_call_is_needed_where_kept(make, drop):
    """The reduced closing call of RK stages 1 and 2 keeps exactly what is
    read before the next opening call: dropping the kept edge fills (boundary
    z faces, IBM stencils on edges) or the kept level jumps (boundary y and z
    faces read the ghost rows) changes the result."""
    case = make()
    ref = _run(case, library_order=False)
    assert np.array_equal(ref[1:], _run(case, library_order=True)[1:])
    orig = Model.__init__

    def patched(self, case, seed):
        orig(self, case, seed)
        if drop == "edges":
            assert self.edge_q.any()
            self.edge_q = np.zeros_like(self.edge_q)
        else:
            assert self.keep_q.any()
            self.keep_q = np.zeros_like(self.keep_q)
    Model.__init__ = patched
    try:
        bad = _run(case, library_order=True)
    finally:
        Model.__init__ = orig
    assert not np.array_equal(ref[1:], bad[1:])


def test_reduced_closing_call_drops_most_of_the_work():
    """On the two-level sphere (boundary cubes away from the level jumps and
    the body) the reduced closing call keeps few tasks and edge fills."""
    case = cases.sphere_ibm(n=8, coarse=2.0, box=((-4, 6), (-4, 4), (-4, 4)),
                            refine_box=((-2, 2), (-2, 2), (-2, 2)))
    tasks, _, _, _, keep_q, edge_q = _plan(case)
    level = tasks[:, 3] != 0
    assert level.sum() > 0
    assert keep_q.sum() < level.sum() // 2
    assert edge_q.sum() < (case.ncube - 1) // 2


def _beside(case):
    lists = [np.ascontiguousarray(a, np.int32) for a in case.bc_lists()]
    ptrs = (C.c_void_p * 6)(*[a.ctypes.data if len(a) else None for a in lists])
    counts = (C.c_int * 6)(*[len(a) for a in lists])
    t = [(None, None, 0) if x is None else
         (np.ascontiguousarray(x[1], np.int32), np.ascontiguousarray(x[2], np.int32),
          (len(x[1]) - 1) // 4) for x in (case.ibm_minus, case.ibm_plus)]
    out = np.zeros(1, np.int32)
    r = lib().bcmg_ghost_beside_plan(
        case.n, case.ncube, C.cast(ptrs, C.c_void_p), C.cast(counts, C.c_void_p),
        None if t[0][0] is None else t[0][0].ctypes.data,
        None if t[0][1] is None else t[0][1].ctypes.data, t[0][2],
        None if t[1][0] is None else t[1][0].ctypes.data,
        None if t[1][1] is None else t[1][1].ctypes.data, t[1][2],
        np.array([1, case.ncube], np.int32), 1, out)
    assert r == 1
    return bool(out[0])


@pytest.mark.parametrize("make", [
    lambda: cases.sphere_ibm(n=8, coarse=2.0, box=((-2, 4), (-2, 2), (-2, 2)),
                             refine_box=((-2, 2), (-2, 2), (-2, 2))),
    lambda: cases.sphere_ibm(n=8, coarse=2.0, box=((-4, 6), (-4, 4), (-4, 4)),
                             refine_box=((-2, 2), (-2, 2), (-2, 2))),
    lambda: cases.random_case(seed=11, n=4, periodic=False),
    lambda: cases.random_case(seed=3, n=8, periodic=True)],
    ids=["sphere_small", "sphere", "random_open_ibm", "random_periodic_ibm"])
def test_ghost_fill_beside_boundary_fill_where_the_plan_allows(make):
    """Where bcmg_ghost_beside_plan lets the IBM ghost fill run beside the
    boundary fill, the two touch disjoint cells: with the ghost fill first
    in every stage the model leaves every cell as the reference's order."""
    case = make()
    if not _beside(case):
        return
    ref = _run(case, library_order=False)
    assert np.array_equal(ref[1:], _run(case, library_order=False, ghost_first=True)[1:])
    assert np.array_equal(ref[1:], _run(case, library_order=True, ghost_first=True)[1:])


def test_ghost_beside_plan_sides():
    """The spheres' IBM cells lie away from their boundary faces (beside);
    the random tables put IBM cells in boundary layers (in order), and there
    the order matters: ghost fill first changes the result."""
    sph = cases.sphere_ibm(n=8, coarse=2.0, box=((-4, 6), (-4, 4), (-4, 4)),
                           refine_box=((-2, 2), (-2, 2), (-2, 2)))
    assert _beside(sph)
    rnd = cases.random_case(seed=11, n=4, periodic=False)
    assert not _beside(rnd)
    # the in-order half of the mixed batch in the GPU on/off comparison
    assert not _beside(cases.random_case(seed=11, n=8, periodic=False, viscous=True))
    assert not np.array_equal(_run(rnd, library_order=False)[1:],
                              _run(rnd, library_order=False, ghost_first=True)[1:])
