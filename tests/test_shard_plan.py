"""Host logic of cube-sharded runs, on CPU with two gloo ranks.

Each rank plans its share of a case on its own (bcmg_shard_plan,
bcmg_shard_bands) and the ranks compare through the process group:

* the ranks' own cubes partition the case;
* for every ordered pair of ranks, the bands the sender computes to pack are
  the bands the receiver computes to unpack (same list, same order);
* a rank's proxies are exactly the source cubes of the bands it receives;
* every face task of a rank's cube that reads a remote cube is covered by a
  band of that cube's face with enough layers (2 for same-level copies and
  injections, 4 for fine -> coarse averages).
"""
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CASES = ("random_open_n4", "two_level_periodic_n4", "two_level_open_n8", "tgv_n8")


def _partitions(case, world):
    """Contiguous halves and a scattered (cube mod world) partition."""
    m = case.ncube - 1
    a = np.zeros(case.ncube, np.int32)
    a[1:] = (np.arange(m) * world) // m
    b = np.zeros(case.ncube, np.int32)
    b[1:] = np.arange(m) % world
    return [a, b]


def _rank(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]
    import torch.distributed as dist
    from bcm_cgli_gb300 import cases
    from golden import golden_cases as G
    dist.init_process_group("gloo")
    out = []
    for name in CASES:
        case = G.golden_cases()[name]
        for rk in _partitions(case, world):
            own, prox = cases.shard_plan(case, rk, rank)
            send = {p: cases.shard_bands(case, rk, rank, p).tolist()
                    for p in range(world) if p != rank}
            recv = {p: cases.shard_bands(case, rk, p, rank).tolist()
                    for p in range(world) if p != rank}
            got = [None] * world
            dist.all_gather_object(got, {"own": own.tolist(), "prox": prox.tolist(),
                                         "send": send, "recv": recv})
            out.append((name, rk.tolist(), got))
    dist.destroy_process_group()
    q.put((rank, out))


def test_two_ranks_plan_the_same_exchange():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 400
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]
    from bcm_cgli_gb300 import _lib
    from golden import golden_cases as G
    L = _lib.lib()
    for (name, rk, got0), (_, _, got1) in zip(res[0], res[1]):
        assert got0 == got1, name  # both ranks gathered the same plans
        case = G.golden_cases()[name]
        rk = np.asarray(rk)
        plans = got0
        owned = sorted(c for pl in plans for c in pl["own"])
        assert owned == list(range(1, case.ncube)), name
        for r, pl in enumerate(plans):
            srcs = set()
            for p, pp in enumerate(plans):
                if p == r:
                    continue
                assert pp["send"][r] == pl["recv"][p], (name, p, r)
                srcs |= {b[0] for b in pl["recv"][p]}
            assert sorted(srcs) == pl["prox"], (name, r)
        # coverage of every cross-rank face task of the global case
        adj = np.ascontiguousarray(case.adj, np.int32)
        csl = np.ascontiguousarray(case.csl, np.int32)
        off = np.zeros(case.ncube + 1, np.int32)
        words = np.zeros(5 * 8 * case.ncube * 6, np.int32)
        nt = L.bcmg_interface_tasks(case.ncube, adj, csl, off, words, 8 * case.ncube * 6)
        assert nt > 0
        words = words[:5 * nt].reshape(nt, 5)
        for c in range(1, case.ncube):
            for t in range(off[c], off[c + 1]):
                src, ax, side, kind = words[t][:4]
                if rk[src] == rk[c] or src == c:
                    continue
                bands = plans[rk[c]]["recv"][rk[src]]
                need = 4 if kind == 2 else 2
                hit = [b for b in bands if b[0] == src and b[1] == ax and b[2] == 1 - side]
                assert hit and hit[0][3] >= need, (name, c, t)


def test_shard_case_refuses_cross_cube_ibm_stencils():
    """A rank fills the IBM ghosts of its own cubes from their own cells; the
    random test tables also reach into other cubes and are refused."""
    sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]
    from bcm_cgli_gb300 import cases
    from golden import golden_cases as G
    case = G.golden_cases()["random_open_n4"]
    rk = np.zeros(case.ncube, np.int32)
    rk[1:] = np.arange(case.ncube - 1) % 2
    with pytest.raises(ValueError):
        cases.shard_case(case, rk, 0)
