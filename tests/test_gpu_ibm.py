"""IBM preprocessing on the GPU (BCM_Immersed_boundary.cpp:127-1081): the
tables and flags equal the oracle's restatement bit for bit, and the
reference-named twin writes the same files as the reference (digests recorded
from it by tests/golden/make_golden.py)."""
import hashlib
import json
import os

import numpy as np
import pytest

import ibm_files
import oracle as O
from bcm_cgli_gb300 import api, cases
from bcm_cgli_gb300._lib import BcmgError
from golden import golden_cases as G

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))["ibm"]
CASES = G.ibm_cases()


@pytest.fixture(scope="module")
def port():
    return O.Port()


def _sha(b):
    return hashlib.sha256(b).hexdigest()


def _equal_tables(a, b):
    for (ga, ia, wa), (gb, ib, wb) in zip(a, b):
        assert np.array_equal(ga, gb) and np.array_equal(ia, ib)
        assert wa.shape == wb.shape and np.array_equal(wa.view(np.int64), wb.view(np.int64))


@pytest.mark.parametrize("name", sorted(CASES))
def test_tables_equal_restatement(port, name):
    case, tris = CASES[name]
    fg, fo = case.fws.copy(), case.fws.copy()
    got = api.ibm_preprocess(case, tris, fg)
    want = port.ibm(case, fo, tris)
    _equal_tables(got, want)
    assert np.array_equal(fg, fo)
    rec = GOLDEN[name]
    assert _sha(ibm_files.text(*got[0]).encode()) == rec["minus"]
    assert _sha(ibm_files.text(*got[1]).encode()) == rec["plus"]
    assert hashlib.sha256(G.canonical(fg)).hexdigest() == rec["fws"]


def _centres(case):
    S = case.n + 4
    dx = (case.cube_size / case.n)[:, None]
    i = np.arange(S)[None, :]
    return [np.ascontiguousarray(case.origin[:, a][:, None] + (i - 1.5) * dx) for a in range(3)]


@pytest.mark.parametrize("name,myid,centres", [("sphere_n8_l5", 0, False),
                                               ("sphere_n8_l2_offset", 3, True)])
def test_twin_writes_reference_files(tmp_path, monkeypatch, name, myid, centres):
    case, tris = CASES[name]
    cases.write_stl(str(tmp_path / "BCM_STL_fine.stl"), tris)
    api.reference_config_for(case)
    monkeypatch.chdir(tmp_path)
    fws = case.fws.copy()
    o = np.ascontiguousarray(case.origin)
    cnt = _centres(case) if centres else [None, None, None]
    api.BCM_Immersed_boundary(myid, case.ncube, 1, None, 0, 0, 0, 0, 0, 0, case.cube_size,
                              case.csl, np.ascontiguousarray(o[:, 0]),
                              np.ascontiguousarray(o[:, 1]), np.ascontiguousarray(o[:, 2]),
                              *cnt, fws, None)
    rec = GOLDEN[name]
    assert _sha((tmp_path / f"IBM_minus{myid:05d}.dat").read_bytes()) == rec["minus"]
    assert _sha((tmp_path / f"IBM_plus{myid:05d}.dat").read_bytes()) == rec["plus"]
    assert hashlib.sha256(G.canonical(fws)).hexdigest() == rec["fws"]


def test_twin_without_stl_file_fails(tmp_path, monkeypatch):
    case, _ = CASES["sphere_n8_l1"]
    api.reference_config_for(case)
    monkeypatch.chdir(tmp_path)
    fws = case.fws.copy()
    o = np.ascontiguousarray(case.origin)
    with pytest.raises(BcmgError, match="BCM_STL_fine.stl"):
        api.BCM_Immersed_boundary(0, case.ncube, 1, None, 0, 0, 0, 0, 0, 0, case.cube_size,
                                  case.csl, np.ascontiguousarray(o[:, 0]),
                                  np.ascontiguousarray(o[:, 1]), np.ascontiguousarray(o[:, 2]),
                                  None, None, None, fws, None)
    assert np.array_equal(fws, case.fws)


def test_no_triangle_near_the_cubes_leaves_everything(port):
    case, _ = CASES["sphere_n8_l1"]
    far = cases.icosphere(1, 0.5, center=(100.0, 0.0, 0.0))
    fws = case.fws.copy()
    (gm, _, _), (gp, _, _) = api.ibm_preprocess(case, far, fws)
    assert len(gm) == 0 and len(gp) == 0 and np.array_equal(fws, case.fws)
    fo = case.fws.copy()
    (om, _, _), (op, _, _) = port.ibm(case, fo, far)
    assert len(om) == 0 and len(op) == 0 and np.array_equal(fo, case.fws)


def test_benchmark_sphere_tables_equal_restatement(port):
    """The sphere benchmark's geometry (1,584 cubes of 16^3 on two levels)
    with the 20,480-triangle body."""
    case = cases.sphere_ibm()
    tris = cases.icosphere(5, 0.5)
    fg, fo = case.fws.copy(), case.fws.copy()
    got = api.ibm_preprocess(case, tris, fg)
    _equal_tables(got, port.ibm(case, fo, tris))
    assert np.array_equal(fg, fo)
    assert len(got[0][0]) + len(got[1][0]) > 500


def test_sphere_case_from_gpu_preprocessing_runs(port):
    """sphere_ibm with the GPU preprocessing gives the same packed tables and
    flags as with the restatement, and a sub-iteration on it is finite."""
    a = cases.sphere_ibm(n=8, box=((-4.0, 6.0), (-4.0, 4.0), (-4.0, 4.0)),
                         refine_box=((-2.0, 2.0), (-2.0, 2.0), (-2.0, 2.0)),
                         preprocess=api.ibm_preprocess, stl_levels=4)
    b = cases.sphere_ibm(n=8, box=((-4.0, 6.0), (-4.0, 4.0), (-4.0, 4.0)),
                         refine_box=((-2.0, 2.0), (-2.0, 2.0), (-2.0, 2.0)),
                         preprocess=lambda c, t: port.ibm(c, c.fws, t), stl_levels=4)
    assert np.array_equal(a.fws, b.fws)
    for x, y in zip(a.ibm_minus + a.ibm_plus, b.ibm_minus + b.ibm_plus):
        assert np.array_equal(np.asarray(x), np.asarray(y))
    ctx = api.CaseContext(a, precision=api.PRECISION_SPLIT)
    ctx.set_state(a.U, a.U, a.U)
    er = ctx.advance(1, 2)
    assert np.isfinite(np.asarray(er)).all()
    ctx.close()
