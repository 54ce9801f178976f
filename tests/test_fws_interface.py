"""The flag field's same-level interface (BCM_FWS_Interface), on the CPU.

* The numpy restatement (oracle.fws_interface) reproduces the digests the
  reference's own compiled routine left on the flag cases
  (tests/golden/golden.json, "flags"), and equals the reference directly on
  more seeds where its sources exist.
* The library's forms equal the restatement bit for bit: the drop-in twin
  BCM_FWS_Interface (the reference's parameter list and same-level lists)
  and bcmg_fws_interface (pairs found from the adjacency).
* Invalid input is rejected with the flags unchanged.
* Two gloo ranks: each packs the flag bands of its cubes for the other,
  unpacks the other's bands into its proxy slots (filled with junk before)
  and runs the routine on its own cubes and proxies; its cubes' flags equal
  those of one process holding the whole case.
"""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

import oracle as O
from bcm_cgli_gb300 import api, cases
from golden import golden_cases as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.json")


def _restated(case):
    return O.fws_interface(case.n, case.ncube, case.csl, case.adj, case.fws)


def _digest(a):
    return hashlib.sha256(G.canonical(a)).hexdigest()


@pytest.fixture(scope="module")
def records():
    with open(GOLDEN) as f:
        return json.load(f)["flags"]


@pytest.mark.parametrize("name", list(G.flag_cases()))
def test_restatement_reproduces_reference_digests(name, records):
    case = G.flag_cases()[name]
    rec = records[name]
    assert _digest(case.fws) == rec["input"]
    out = _restated(case)
    assert _digest(out) == rec["fws"]
    assert int((out != case.fws).sum()) == rec["changed"]


def _more_cases():
    """More seeds on the flag cases' four grids (so the reference compiled
    for those configurations serves them too)."""
    def finest(case):
        case.csl = np.zeros_like(case.csl)
        return case
    out = []
    for s in range(31, 35):
        frac = 0.25 + 0.05 * (s % 4)
        out += [finest(cases.random_case(seed=s, ncx=2, ncy=2, ncz=1, n=8, periodic=s % 2 == 0,
                                         solid_frac=frac, ghost_frac=0.2)),
                finest(cases.random_case(seed=s, ncx=3, ncy=2, ncz=2, n=4, periodic=s % 2 == 1,
                                         solid_frac=frac, ghost_frac=0.2)),
                cases.random_two_level_case(seed=s, n=4, periodic=s % 2 == 0, solid_frac=frac,
                                            ghost_frac=0.2),
                finest(cases.random_case(seed=s, ncx=1, ncy=1, ncz=1, n=4, periodic=True,
                                         solid_frac=frac, ghost_frac=0.2))]
    return out


@pytest.mark.skipif(not O.reference_available(), reason="reference sources not on this host")
def test_restatement_equals_reference_directly():
    for case in _more_cases():
        ref = O.Ref(case)
        a = case.fws.copy()
        ref.fws_interface(case, a)
        assert np.array_equal(a, _restated(case)), case.name


@pytest.mark.parametrize("name", list(G.flag_cases()))
def test_library_forms_equal_restatement(name):
    case = G.flag_cases()[name]
    want = _restated(case)
    twin = case.fws.copy()
    api.reference_config_for(case)
    try:
        api.BCM_FWS_Interface_for_case(case, twin)
    finally:
        api.set_reference_config()
    assert np.array_equal(twin, want)
    lib_form = case.fws.copy()
    api.fws_interface(case.n, case.ncube, case.csl, case.adj, lib_form)
    assert np.array_equal(lib_form, want)


def test_library_form_on_more_cases():
    for case in _more_cases():
        f = case.fws.copy()
        api.fws_interface(case.n, case.ncube, case.csl, case.adj, f)
        assert np.array_equal(f, _restated(case)), case.name


def test_invalid_input_leaves_flags_unchanged():
    case = G.flag_cases()["flags_two_level_n4"]
    X, Y, Z = (lst[0] for lst in api.interface_lists(case))
    api.reference_config_for(case)
    try:
        # cross-rank lists on one process
        f = case.fws.copy()
        with pytest.raises(api.BcmgError, match="cross-rank"):
            api.BCM_FWS_Interface(0, case.ncube, 1, 1, 0, len(X) - 1, len(Y) - 1, len(Z) - 1,
                                  case.csl, case.adj, X, Y, Z, f)
        assert np.array_equal(f, case.fws)
        # a same-level pair whose cubes the level array puts on two levels
        c = int(X[1])
        c2 = int(case.adj[c, 1, 2])
        csl = case.csl.copy()
        csl[c2] = csl[c] + 1
        with pytest.raises(api.BcmgError, match="differ in level"):
            api.BCM_FWS_Interface(0, case.ncube, 1, 0, 0, len(X) - 1, len(Y) - 1, len(Z) - 1,
                                  csl, case.adj, X, Y, Z, f)
        assert np.array_equal(f, case.fws)
        # a listed cube without a +x neighbour in slot 1
        adj = case.adj.copy()
        adj[c, 1, 2] = 0
        with pytest.raises(api.BcmgError, match="no neighbour"):
            api.BCM_FWS_Interface(0, case.ncube, 1, 0, 0, len(X) - 1, len(Y) - 1, len(Z) - 1,
                                  case.csl, adj, X, Y, Z, f)
        assert np.array_equal(f, case.fws)
    finally:
        api.set_reference_config()
    adj = case.adj.copy()
    adj[1, 2, 4] = case.ncube  # out of range
    with pytest.raises(api.BcmgError, match="out of range"):
        api.fws_interface(case.n, case.ncube, case.csl, adj, f)
    assert np.array_equal(f, case.fws)


def test_band_pack_unpack_round_trip():
    case = G.flag_cases()["flags_open_n4"]
    n = case.n
    bands = np.array([[1, 0, 1, 2], [2, 1, 0, 2], [5, 2, 1, 4], [3, 0, 0, 1]], np.int32)
    buf = api.fws_band_pack(n, case.fws, bands)
    assert len(buf) == (2 + 2 + 4 + 1) * n * n
    # first band: cube 1, x axis, high side, layers n, n+1; (layer, y, z) order
    assert np.array_equal(buf[:2 * n * n].reshape(2, n, n), case.fws[1, n:n + 2, 2:n + 2, 2:n + 2])
    f = np.full_like(case.fws, 9)
    api.fws_band_unpack(n, f, bands, buf)
    inside = np.zeros(case.fws.shape, bool)
    for c, ax, side, L in bands:
        sl = [c, slice(2, n + 2), slice(2, n + 2), slice(2, n + 2)]
        sl[1 + ax] = slice(n + 2 - L, n + 2) if side else slice(2, 2 + L)
        assert np.array_equal(f[tuple(sl)], case.fws[tuple(sl)])
        inside[tuple(sl)] = True
    assert (f[~inside] == 9).all()  # nothing outside the bands is written
    with pytest.raises(api.BcmgError, match="invalid"):
        api.fws_band_pack(n, case.fws, [[case.ncube, 0, 0, 2]])


# ---------------------------------------------------------------------------
# two ranks
# ---------------------------------------------------------------------------
SHARD_CASES = ("flags_periodic_n8", "flags_open_n4", "flags_two_level_n4")


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]
    import torch
    import torch.distributed as dist
    from bcm_cgli_gb300 import api, cases
    from golden import golden_cases as G
    dist.init_process_group("gloo")
    out = []
    for name in SHARD_CASES:
        case = G.flag_cases()[name]
        case.ibm_minus = case.ibm_plus = None  # not read by the flag routine
        m = case.ncube - 1
        rk = np.zeros(case.ncube, np.int32)
        rk[1:] = np.arange(m) % world
        sub, own, prox = cases.shard_case(case, rk, rank)
        g2l = {int(g): i + 1 for i, g in enumerate(list(own) + list(prox))}
        fws = sub.fws.copy()
        fws[1 + len(own):] = 5  # proxies: only what the bands bring is known
        for p in range(world):
            if p == rank:
                continue
            send = cases.shard_bands(case, rk, rank, p).copy()
            recv = cases.shard_bands(case, rk, p, rank).copy()
            send[:, 0] = [g2l[int(g)] for g in send[:, 0]]
            recv[:, 0] = [g2l[int(g)] for g in recv[:, 0]]
            mine = torch.from_numpy(api.fws_band_pack(sub.n, fws, send))
            theirs = torch.zeros(int(recv[:, 3].sum()) * sub.n ** 2, dtype=torch.int32)
            # lower rank sends first
            if rank < p:
                dist.send(mine, p)
                dist.recv(theirs, p)
            else:
                dist.recv(theirs, p)
                dist.send(mine, p)
            api.fws_band_unpack(sub.n, fws, recv, theirs.numpy())
        api.fws_interface(sub.n, sub.ncube, sub.csl, sub.adj, fws)
        out.append((name, own.tolist(), fws[1:1 + len(own)].copy()))
    dist.destroy_process_group()
    q.put((rank, out))


def test_two_ranks_exchange_flag_bands():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 28100 + os.getpid() % 800  # a range no other test uses
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=180) for _ in range(2))
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    for rank in range(2):
        for name, own, got in res[rank]:
            case = G.flag_cases()[name]
            want = _restated(case)
            assert np.array_equal(got, want[own]), (name, rank)


def test_synthetic_sphere_flags_against_the_setup_routine():
    """What the routine would change on the benchmark's sphere grids after
    their IBM preprocessing (main.cpp:1070 runs it there; the synthetic
    builders do not): nothing on the 1,584-cube sphere, and 312 ghost-layer
    flags next to the body on the batch's grids (fine cubes of edge 0.5),
    240 fluid -> ghost and 72 ghost -> fluid."""
    port = O.Port()

    def pre(case, tris):
        return port.ibm(case, case.fws, tris)
    single = cases.sphere_ibm(preprocess=pre)
    assert np.array_equal(_restated(single), single.fws)
    grid = cases.sphere_cubes(64, preprocess=pre)  # the body's 64 fine cubes of every batch case
    out = _restated(grid)
    changed = np.argwhere(out != grid.fws)
    n = grid.n
    assert len(changed) == 312
    assert all(min(x[1:]) < 2 or max(x[1:]) > n + 1 for x in changed)  # ghost layers only
    before, after = grid.fws[tuple(changed.T)], out[tuple(changed.T)]
    assert int(((before == 1) & (after == 0)).sum()) == 240
    assert int(((before == 0) & (after == 1)).sum()) == 72
