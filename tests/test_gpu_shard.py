"""Cube-sharded runs on one GPU against one context holding every cube.

api.ShardedRun gives every rank its own context (its cubes, then proxies
of the remote cubes its face tasks read) and host thread; the exchange hook
moves the face bands through device buffers and adds the ranks' norm sums.
After whole dual-time steps every cube's cells (ghost layers included) must
equal the single context's bit for bit, FP64 and split precision, RK and
LU-SGS sub-iterations, two and three ranks, contiguous and scattered
partitions; the norms agree to 1e-12 (the ranks' sums are added in another
order than one context's blocks).  The two force sums (drag, lift) are sums
of surface terms of both signs, so a near-zero lift is held to 1e-12 of the
larger force magnitude rather than of itself.
"""
import numpy as np
import pytest

from bcm_cgli_gb300 import api, cases
from golden import golden_cases as G

pytestmark = pytest.mark.gpu

NORM_RTOL = 1e-12


def _norms_close(a, b):
    a, b = np.asarray(a), np.asarray(b)
    for m in range(1, 6):
        assert abs(a[m] - b[m]) <= NORM_RTOL * max(abs(a[m]), 1e-300), (m, a, b)
    force = max(abs(a[6]), abs(a[7]), 1e-300)
    for m in (6, 7):
        assert abs(a[m] - b[m]) <= NORM_RTOL * force, (m, a, b)


def _same_cube(t):
    """The IBM entries whose image-point stencil lies in the ghost's own cube
    (the random test tables also cross cubes, which real tables never do and
    sharded runs refuse)."""
    if t is None:
        return None
    W, Gi, I = t
    m = (len(Gi) - 1) // 4
    keep = Gi[1:].reshape(m, 4)[:, 0] == I[1:].reshape(m, 4)[:, 0]
    return (np.concatenate([W[:1], W[1:].reshape(m, 8)[keep].reshape(-1)]),
            np.concatenate([Gi[:1], Gi[1:].reshape(m, 4)[keep].reshape(-1)]).astype(np.int32),
            np.concatenate([I[:1], I[1:].reshape(m, 4)[keep].reshape(-1)]).astype(np.int32))


def _case(name):
    if name == "sphere_two_level":
        return cases.sphere_ibm(n=8, coarse=2.0, box=((-2, 4), (-2, 2), (-2, 2)),
                                refine_box=((-2, 2), (-2, 2), (-2, 2)))
    case = G.golden_cases()[name]
    case.ibm_minus, case.ibm_plus = _same_cube(case.ibm_minus), _same_cube(case.ibm_plus)
    return case


def _ranks(case, nrank, scattered):
    rk = np.zeros(case.ncube, np.int32)
    m = case.ncube - 1
    rk[1:] = np.arange(m) % nrank if scattered else (np.arange(m) * nrank) // m
    return rk


@pytest.mark.parametrize("name", ["tgv_n8", "two_level_open_n8", "random_open_n4",
                                  "sphere_two_level"])
@pytest.mark.parametrize("precision", [api.PRECISION_FP64, api.PRECISION_SPLIT])
@pytest.mark.parametrize("nrank,scattered", [(2, False), (3, True)])
def test_sharded_run_equals_one_context(name, precision, nrank, scattered):
    case = _case(name)
    one = api.CaseContext(case, precision=precision)
    one.set_state(case.U, case.U, case.U)
    er1 = one.advance(2, 2, use_graph=False)
    ref = one.get_state()
    one.close()
    sh = api.ShardedRun(case, _ranks(case, nrank, scattered), precision=precision)
    sh.set_state(case.U, case.U, case.U)
    er2 = sh.advance(2, 2)
    got = sh.get_state()
    sh.close()
    for k, a, b in zip(("U1_", "U1", "U1q"), ref, got):
        bad = np.argwhere(a[1:] != b[1:])
        assert bad.size == 0, f"{name} {k}: {len(bad)} mismatches, first {bad[:3]}"
    _norms_close(er1, er2)


@pytest.mark.parametrize("precision", [api.PRECISION_FP64, api.PRECISION_SPLIT])
def test_sharded_lusgs_equals_one_context(precision):
    case = _case("two_level_open_n8")
    one = api.CaseContext(case, precision=precision)
    one.set_method(api.METHOD_LUSGS)
    one.set_state(case.U, case.U, case.U)
    one.advance(1, 3, use_graph=False)
    ref = one.get_state()
    one.close()
    sh = api.ShardedRun(case, _ranks(case, 2, True), precision=precision)
    for c in sh.ctx:
        c.set_method(api.METHOD_LUSGS)
    sh.set_state(case.U, case.U, case.U)
    sh.advance(1, 3)
    got = sh.get_state()
    sh.close()
    for a, b in zip(ref, got):
        assert np.array_equal(a[1:], b[1:])


def test_sharded_context_refuses_graphs():
    case = _case("tgv_n8")
    sh = api.ShardedRun(case, _ranks(case, 2, False))
    with pytest.raises(api.BcmgError):
        sh.ctx[0].advance(1, 1, use_graph=True)
    sh.close()


def _dist_rank(rank, world, port, name, precision, q):
    import os
    import sys
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "tests"), os.path.join(root, "oracle")]
    import torch.distributed as dist
    from bcm_cgli_gb300 import api as A
    dist.init_process_group("gloo")
    case = _case(name)
    sh = A.DistShard(case, _ranks(case, world, True), precision=precision)
    sh.set_state(case.U, case.U, case.U)
    er = sh.advance(2, 2)
    own, u, u1, uq = sh.own_state()
    sh.close()
    dist.destroy_process_group()
    q.put((rank, own, u, u1, uq, er))


@pytest.mark.parametrize("precision", [api.PRECISION_FP64, api.PRECISION_SPLIT])
def test_two_processes_over_gloo_equal_one_context(precision):
    """Two processes, each a rank of the sharded run on this GPU, exchanging
    through torch.distributed (gloo, host-staged): the same bits as one
    context."""
    import os

    import torch.multiprocessing as mp
    name = "two_level_open_n8"
    case = _case(name)
    one = api.CaseContext(case, precision=precision)
    one.set_state(case.U, case.U, case.U)
    er1 = one.advance(2, 2, use_graph=False)
    ref = one.get_state()
    one.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29900 + os.getpid() % 90
    ps = [ctx.Process(target=_dist_rank, args=(r, 2, port, name, precision, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = [q.get(timeout=600) for _ in range(2)]
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    for rank, own, u, u1, uq, er in res:
        for a, b in zip(ref, (u, u1, uq)):
            assert np.array_equal(a[own], b)
        _norms_close(er1, er)
