"""CPU tests of the host-side logic and of the C ABI surface (no GPU calls)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import oracle as O
from bcm_cgli_gb300 import cases
from bcm_cgli_gb300._lib import LIB_PATH, lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if not fn.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", fn)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", src,
                             flags=re.M):
            if m.group(1) not in ("if", "defined") and \
                    not m.group(0).lstrip().startswith("typedef"):
                names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol():
    assert os.path.isfile(LIB_PATH), "build the library first (__graft_entry__.build())"
    L = C.CDLL(LIB_PATH)
    names = _header_functions()
    assert {"BCM_Flux_XYZ_Viscous_Runge_kutta", "BCM_Interface", "bcmg_case_create"} <= names
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing


def test_reference_config_roundtrip():
    from bcm_cgli_gb300 import api
    api.set_reference_config(ncube_x=24, mpi_ncube=512, mu_L=0.0256, rho0=1.2, U0=34.6,
                             Uin=34.6, P0=101300.0)
    from bcm_cgli_gb300._lib import RefConfig
    c = RefConfig()
    lib().bcmg_get_reference_config(C.byref(c))
    assert (c.ncube_x, c.mpi_ncube, c.mu_L) == (24, 512, 0.0256)
    with pytest.raises(Exception):
        api.set_reference_config(ncube_x=6)  # not a multiple of 4


def _ibm_levels(case, table):
    W, G, I = table
    nbc = (len(G) - 1) // 4
    lev = np.zeros(nbc, np.int32)
    nl = lib().bcmg_ibm_schedule(nbc, np.ascontiguousarray(G, np.int32),
                                 np.ascontiguousarray(I, np.int32), case.n, case.ncube, lev)
    return nl, lev


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_ibm_levels_reproduce_the_serial_loop(seed):
    """Applying the ghost entries level by level (any order inside a level)
    gives the reference's serial result bit for bit: run the oracle's serial
    loop on the level-sorted table (reversed inside each level) and compare."""
    case = cases.random_case(seed=seed, n=4)
    W, G, I = case.ibm_minus
    nl, lev = _ibm_levels(case, case.ibm_minus)
    assert nl >= 1 and lev.min() >= 1
    nbc = len(lev)
    order = sorted(range(nbc), key=lambda e: (lev[e], -e))
    W2 = np.concatenate([[0.0]] + [W[8 * e + 1:8 * e + 9] for e in order])
    G2 = np.concatenate([[0]] + [G[4 * e + 1:4 * e + 5] for e in order]).astype(np.int32)
    I2 = np.concatenate([[0]] + [I[4 * e + 1:4 * e + 5] for e in order]).astype(np.int32)
    port = O.Port()
    a, b = O.State(case), O.State(case)
    port.ghost(case, a.U1_, -1)
    case2 = cases.random_case(seed=seed, n=4)
    case2.ibm_minus = (W2, G2, I2)
    port.ghost(case2, b.U1_, -1)
    assert np.array_equal(a.U1_, b.U1_)


def test_ibm_levels_reject_out_of_range_indices():
    case = cases.random_case(seed=1, n=4)
    W, G, I = case.ibm_minus
    I = I.copy()
    I[4] = case.S - 1  # k + 1 would leave the padded cube
    nl, _ = _ibm_levels(case, (W, G, I))
    assert nl == -1


def test_interface_tasks_match_reference_lists():
    """Face tasks from adjacency equal the same-level pairs the reference's
    BCM_Interface_table.cpp would list (periodic box: 6 faces per cube)."""
    case = cases.taylor_green(ncx=3, n=4)
    off = np.zeros(case.ncube + 1, np.int32)
    words = np.zeros(5 * 6 * case.ncube, np.int32)
    nt = lib().bcmg_interface_tasks(case.ncube, np.ascontiguousarray(case.adj, np.int32),
                                    case.csl, off, words, 6 * case.ncube)
    assert nt == 6 * (case.ncube - 1)
    w = words[:5 * nt].reshape(-1, 5)
    for c in range(1, case.ncube):
        t = w[off[c]:off[c + 1]]
        assert len(t) == 6
        for src, ax, side, kind, slot in t:
            assert kind == 0
            # side 0: low ghosts from the -axis neighbour; 1: high from +axis
            assert src == case.adj[c, 1, 1 + 2 * ax + side]


def test_open_box_interface_tasks_skip_domain_faces():
    ncube, cs, csl, org, adj = cases.open_box(2, 2, 2, 4, 1.0)
    off = np.zeros(ncube + 1, np.int32)
    words = np.zeros(5 * 6 * ncube, np.int32)
    nt = lib().bcmg_interface_tasks(ncube, np.ascontiguousarray(adj, np.int32),
                                    np.ascontiguousarray(csl, np.int32), off, words, 6 * ncube)
    assert nt == 3 * (ncube - 1)  # each cube of a 2x2x2 open box has 3 neighbours


def test_two_level_interface_tasks():
    """A refined coarse cube in a periodic 2x2x2 coarse box: every face of the
    8 fine cubes that touches a coarse cube gets one coarse->fine task; each
    coarse face next to the refined block gets four fine->coarse quadrant
    tasks (slots 1..4)."""
    case = cases.random_two_level_case(seed=1, n=4)
    off = np.zeros(case.ncube + 1, np.int32)
    words = np.zeros(5 * 24 * case.ncube, np.int32)
    nt = lib().bcmg_interface_tasks(case.ncube, np.ascontiguousarray(case.adj, np.int32),
                                    case.csl, off, words, 24 * case.ncube)
    assert nt > 0
    w = words[:5 * nt].reshape(-1, 5)
    kinds = np.bincount(w[:, 3], minlength=3)
    fine = [c for c in range(1, case.ncube) if case.csl[c] == 0]
    # each fine cube: 3 of its 6 faces touch coarse cubes (periodic 2x2x2 box)
    assert kinds[1] == 3 * len(fine)
    # each coarse face adjoining the refined block: 4 quadrant tasks
    assert kinds[2] % 4 == 0 and kinds[2] > 0
    for c in range(1, case.ncube):
        t = w[off[c]:off[c + 1]]
        faces = {}
        for src, ax, side, kind, slot in t:
            faces.setdefault((ax, side), []).append((kind, slot))
        for f, ks in faces.items():
            assert (len(ks) == 1 and ks[0][0] in (0, 1)) or sorted(ks) == [(2, s) for s in (1, 2, 3, 4)]


def test_level_jump_beyond_2_to_1_is_rejected():
    case = cases.random_two_level_case(seed=1, n=4)
    csl = case.csl.copy()
    csl[csl == 1] = 3  # make the coarse cubes 8x the fine size
    off = np.zeros(case.ncube + 1, np.int32)
    words = np.zeros(5 * 24 * case.ncube, np.int32)
    nt = lib().bcmg_interface_tasks(case.ncube, np.ascontiguousarray(case.adj, np.int32), csl,
                                    off, words, 24 * case.ncube)
    assert nt == -1


def _plan(case):
    """bcmg_interface_plan of a case: (tasks [t, 5], destination cube per
    task, keep_prologue, push table [ncube, 6], return code)."""
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
    gcs = []
    for t in (case.ibm_minus, case.ibm_plus):
        g = None if t is None else np.ascontiguousarray(t[1], np.int32)
        gcs.append((g, 0 if g is None else (len(g) - 1) // 4))
    keep = np.zeros(max(nt, 1), np.int32)
    push = np.zeros(6 * case.ncube, np.int32)
    r = lib().bcmg_interface_plan(case.n, case.ncube, adj, csl, C.cast(ptrs, C.c_void_p),
                                  C.cast(counts, C.c_void_p),
                                  None if gcs[0][0] is None else gcs[0][0].ctypes.data, gcs[0][1],
                                  None if gcs[1][0] is None else gcs[1][0].ctypes.data, gcs[1][1],
                                  keep, push, cap)
    dst = np.repeat(np.arange(case.ncube), np.diff(off))
    return words[:5 * nt].reshape(-1, 5), dst, keep[:nt], push.reshape(case.ncube, 6), r


def _prologue_rule(case, tasks, dst):
    """Restatement of the opening-call rule: a level jump, a face the
    boundary fill writes, or a face whose ghost layers (destination) or
    copied interior layers (source) hold an IBM ghost cell."""
    n = case.n
    mask = np.zeros(case.ncube, np.int64)
    for bit, lst in enumerate(case.bc_lists()):
        for c in lst:
            mask[c] |= 1 << bit
    gc = set()
    for t in (case.ibm_minus, case.ibm_plus):
        if t is not None:
            g = np.asarray(t[1][1:]).reshape(-1, 4)
            gc |= {tuple(int(v) for v in row) for row in g}

    def holds(cube, ax, layers):
        for (g, *x) in gc:
            if g == cube and x[ax] in layers and all(
                    2 <= x[a] <= n + 1 for a in range(3) if a != ax):
                return True
        return False

    out = []
    for (src, ax, side, kind, slot), c in zip(tasks, dst):
        dl = (0, 1) if side == 0 else (n + 2, n + 3)
        sl = (n, n + 1) if side == 0 else (2, 3)
        out.append(int(kind != 0 or (mask[c] >> (2 * ax + side)) & 1 or holds(c, ax, dl)
                       or holds(src, ax, sl)))
    return np.array(out, np.int32)


def test_prologue_plan_periodic_box_keeps_box_faces():
    """Periodic 4x4x4 box (the boundary fill runs on box faces before the
    periodic copy overwrites it): the opening call keeps exactly the tasks
    whose destination face lies on the box boundary, 96 of 384."""
    case = cases.taylor_green(ncx=4, n=4)
    tasks, dst, keep, push, r = _plan(case)
    assert r == len(tasks) == 384
    assert keep.sum() == 96
    assert np.array_equal(keep, _prologue_rule(case, tasks, dst))


@pytest.mark.parametrize("make", [
    lambda: cases.random_two_level_case(seed=6, n=8, periodic=False),
    lambda: cases.random_two_level_case(seed=1, n=4),
    lambda: cases.random_case(seed=3, n=8, periodic=True),
    lambda: cases.sphere_ibm(n=8, coarse=2.0, box=((-2, 4), (-2, 2), (-2, 2)),
                             refine_box=((-2, 2), (-2, 2), (-2, 2)))])
def test_prologue_plan_matches_rule(make):
    """Level jumps, boundary faces and faces touching IBM ghost cells are
    kept, nothing else; the push table has one slot per same-level task,
    pointing at its destination, and none for level jumps."""
    case = make()
    tasks, dst, keep, push, r = _plan(case)
    assert r == len(tasks)
    assert np.array_equal(keep, _prologue_rule(case, tasks, dst))
    assert keep.sum() < len(tasks)
    same = tasks[:, 3] == 0
    assert np.count_nonzero(push) == np.count_nonzero(same)
    for (src, ax, side, kind, slot), c in zip(tasks[same], dst[same]):
        assert push[src, 2 * ax + (0 if side == 1 else 1)] == c


def test_interface_plan_error_codes():
    """-2 when the task buffer is too small, -1 for invalid input."""
    case = cases.taylor_green(ncx=2, n=4)
    adj = np.ascontiguousarray(case.adj, np.int32)
    csl = np.ascontiguousarray(case.csl, np.int32)
    lists = [np.ascontiguousarray(a, np.int32) for a in case.bc_lists()]
    ptrs = (C.c_void_p * 6)(*[a.ctypes.data if len(a) else None for a in lists])
    counts = (C.c_int * 6)(*[len(a) for a in lists])
    keep = np.zeros(64, np.int32)
    push = np.zeros(6 * case.ncube, np.int32)

    def plan(ncube, adj_, cap):
        return lib().bcmg_interface_plan(case.n, ncube, adj_, csl, C.cast(ptrs, C.c_void_p),
                                         C.cast(counts, C.c_void_p), None, 0, None, 0, keep,
                                         push, cap)
    assert plan(case.ncube, adj, 64) == 6 * (case.ncube - 1)
    assert plan(case.ncube, adj, 10) == -2
    bad = adj.copy()
    bad[1, 1, 2] = case.ncube + 3
    assert plan(case.ncube, bad, 64) == -1
    assert plan(1, adj, 64) == -1


def _create_error(case_list, precision=0):
    """bcmg_case_create / bcmg_batch_create of invalid descriptors: they fail
    in the host validation, before any device work (so on a CPU too)."""
    from bcm_cgli_gb300 import api
    try:
        if len(case_list) == 1:
            api.CaseContext(case_list[0], precision=precision)
        else:
            api.BatchContext(case_list, precision=precision)
    except api.BcmgError as e:
        return str(e)
    return None


def test_invalid_descriptors_rejected_on_the_host():
    good = cases.random_case(seed=3, n=4)

    def variant(**kw):
        c = cases.random_case(seed=3, n=4)
        for k, v in kw.items():
            setattr(c, k, v)
        return c

    adj = good.adj.copy()
    adj[1, 1, 2] = good.ncube + 5  # neighbour outside the cube list
    assert _create_error([variant(adj=adj)]) is not None
    cs = good.cube_size.copy()
    cs[2] = 0.0
    assert "cube_size" in _create_error([variant(cube_size=cs)])
    assert "n must be a multiple of 4" in _create_error([variant(n=6)])
    assert "precision" in _create_error([good], precision=7)
    two = cases.random_two_level_case(seed=1, n=4)
    csl = two.csl.copy()
    csl[csl == 1] = 3  # an 8:1 jump between neighbours
    two.csl = csl
    assert "2:1" in _create_error([two])
    # a batch needs one n and one precision across its cases
    other = cases.random_case(seed=4, n=8)
    assert "same n" in _create_error([good, other])


@pytest.mark.skipif(not O.reference_available(), reason="reference sources not on this host")
def test_reference_shim_compiles_against_main_h(tmp_path):
    """The C++ shim provides exactly the signatures the reference's main.h
    declares (compile-only check against the reference's own header)."""
    src = tmp_path / "shim.cpp"
    src.write_text('#include "Resolution.h"\n#include "main.h"\n'
                   '#include "bcm_gb300_reference_shim.hpp"\n')
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-w",
                        "-I", O.ref_build.REF_DIR, "-I", os.path.join(ROOT, "include"),
                        "-I", os.path.join(ROOT, "oracle", "mpi_stub"), str(src)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


SHIM_ROUTINES = ("BCM_Flux_XYZ_Viscous_Runge_kutta", "BCM_X_boundary_condition",
                 "BCM_Y_boundary_condition", "BCM_Z_boundary_condition", "BCM_Ghostcell_minus",
                 "BCM_Ghostcell_plus", "BCM_Interface", "BCM_Immersed_boundary",
                 "BCM_FWS_Interface")


@pytest.mark.skipif(not O.reference_available(), reason="reference sources not on this host")
def test_reference_shim_defines_main_h_symbols(tmp_path):
    """A signature that differs from main.h would only add an overload; so a
    caller compiled against main.h alone takes the address of every replaced
    routine, and the shim's object must define each C++ symbol it needs."""
    inc = ["-I", O.ref_build.REF_DIR, "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle", "mpi_stub")]
    caller = tmp_path / "caller.cpp"
    caller.write_text('#include "Resolution.h"\n#include "main.h"\nvoid *routines[] = {' +
                      ", ".join(f"(void *)&{f}" for f in SHIM_ROUTINES) + "};\n")
    shim = tmp_path / "shim.cpp"
    shim.write_text('#include "Resolution.h"\n#include "main.h"\n'
                    '#include "bcm_gb300_reference_shim.hpp"\n')
    syms = {}
    for src in (caller, shim):
        obj = src.with_suffix(".o")
        r = subprocess.run(["g++", "-std=c++17", "-c", "-w", *inc, str(src), "-o", str(obj)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-2000:]
        out = subprocess.run(["nm", str(obj)], capture_output=True, text=True).stdout
        syms[src.name] = [line.split() for line in out.splitlines()]
    needed = {s[-1] for s in syms["caller.cpp"] if s[-2] == "U" and "BCM_" in s[-1]}
    defined = {s[-1] for s in syms["shim.cpp"] if s[-2] == "T"}
    assert len(needed) == len(SHIM_ROUTINES)
    assert needed <= defined, sorted(needed - defined)


def test_batch_create_rejects_mismatched_cases_before_touching_the_gpu():
    """bcmg_batch_create validates every case on the host first: different n,
    out-of-range adjacency and boundary entries are refused with an error
    naming the case, before any device work."""
    import ctypes as C
    from bcm_cgli_gb300 import _lib, api
    a = cases.random_case(seed=1, n=4, periodic=True)
    b = cases.random_case(seed=2, n=8, periodic=True)
    keep = []
    descs = (_lib.CaseDesc * 2)(api._case_desc(a, 0, keep), api._case_desc(b, 0, keep))
    h = C.c_void_p()
    L = _lib.lib()
    assert L.bcmg_batch_create(2, descs, C.byref(h)) != 0
    assert "case 1" in _lib.last_error() and "same n" in _lib.last_error()
    c = cases.random_case(seed=3, n=4, periodic=False)
    bad_adj = c.adj.copy()
    bad_adj[1, 1, 2] = c.ncube + 5
    c.adj = bad_adj
    descs = (_lib.CaseDesc * 2)(api._case_desc(a, 0, keep), api._case_desc(c, 0, keep))
    assert L.bcmg_batch_create(2, descs, C.byref(h)) != 0
    assert "case 1" in _lib.last_error() and "adj_number" in _lib.last_error()
    assert L.bcmg_batch_create(0, descs, C.byref(h)) != 0
