"""PLOT3D output on the GPU (BCM_Output.cpp:16-300): the files are
byte-identical to the oracle's restatement, which is pinned to the
reference's own writer (tests/test_oracle_golden.py); the solution write is
a snapshot that the solver may overtake."""
import os

import numpy as np
import pytest

import oracle as O
import plot3d
from bcm_cgli_gb300 import api, cases
from golden import golden_cases as G

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["random_open_n4", "two_level_open_n8"])
def test_output_bytes_equal_oracle(tmp_path, name):
    case = G.golden_cases()[name]
    ctx = api.CaseContext(case)
    ctx.set_state(case.U, case.U, case.U)
    ctx.advance(1, 2)
    U1_ = ctx.get_state()[0]
    qf, xf = tmp_path / "q.q", tmp_path / "g.x"
    ctx.output_q(str(qf), ncube_out=case.phys.mpi_ncube)
    ctx.output_wait()
    ctx.output_x(str(xf), case.origin, ncube_out=case.phys.mpi_ncube)
    assert qf.read_bytes() == plot3d.solution_bytes(case.n, U1_, case.phys.mpi_ncube)
    assert xf.read_bytes() == plot3d.grid_bytes(case.n, case.ncube, case.cube_size, case.origin,
                                                case.phys.mpi_ncube)
    ctx.close()


def test_output_is_a_snapshot_the_solver_may_overtake(tmp_path):
    case = cases.taylor_green(ncx=4, n=16)  # 64 cubes of 16^3
    ctx = api.CaseContext(case, precision=api.PRECISION_SPLIT)
    ctx.set_state(case.U, case.U, case.U)
    ctx.advance(1, 2)
    before = ctx.get_state()[0]
    ctx.output_q(str(tmp_path / "a.q"))
    ctx.advance(2, 3)  # queued behind the snapshot, runs while the file is written
    ctx.output_wait()
    after = ctx.get_state()[0]
    assert not np.array_equal(before, after)
    assert (tmp_path / "a.q").read_bytes() == plot3d.solution_bytes(case.n, before, case.ncube - 1)
    ctx.close()


def test_output_per_case_of_a_batch(tmp_path):
    cs = [cases.random_case(seed=4, n=8, periodic=True), cases.taylor_green(ncx=2, n=8)]
    b = api.BatchContext(cs)
    for q, c in enumerate(cs):
        b.set_case_state(q, c.U, c.U, c.U)
    b.advance(1, 1)
    for q, c in enumerate(cs):
        U1_ = b.get_case_state(q)[0]
        b.output_q(str(tmp_path / f"c{q}.q"), q=q)
        b.output_x(str(tmp_path / f"c{q}.x"), c.origin, q=q)
        b.output_wait()
        assert (tmp_path / f"c{q}.q").read_bytes() == plot3d.solution_bytes(c.n, U1_, c.ncube - 1)
        assert (tmp_path / f"c{q}.x").read_bytes() == plot3d.grid_bytes(
            c.n, c.ncube, c.cube_size, c.origin, c.ncube - 1)
    b.close()


def test_output_large_file_in_chunks(tmp_path):
    """More than one pinned chunk (32 MB) per file."""
    case = cases.taylor_green(ncx=6, n=24)  # 216 cubes: 190 MB solution file
    ctx = api.CaseContext(case, precision=api.PRECISION_SPLIT)
    ctx.set_state(case.U, case.U, case.U)
    ctx.output_q(str(tmp_path / "big.q"))
    ctx.output_wait()
    data = (tmp_path / "big.q").read_bytes()
    assert data == plot3d.solution_bytes(case.n, case.U, case.ncube - 1)
    ctx.close()
