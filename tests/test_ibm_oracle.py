"""The IBM preprocessing restatement (oracle/bcm_oracle_ibm.c) pinned to the
reference's BCM_Immersed_boundary: its table files and flags against the
digests tests/golden/make_golden.py recorded from the compiled reference,
and, where the reference sources exist, against the reference directly."""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(HERE, "golden"), os.path.join(os.path.dirname(HERE), "oracle")]

import ibm_files  # noqa: E402
import oracle as O  # noqa: E402
from golden_cases import canonical, ibm_cases  # noqa: E402

from bcm_cgli_gb300 import cases  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "golden.json")))["ibm"]
CASES = ibm_cases()


@pytest.fixture(scope="module")
def port():
    return O.Port()


def _sha(b):
    return hashlib.sha256(b).hexdigest()


@pytest.mark.parametrize("name", sorted(CASES))
def test_restatement_matches_reference_files(port, name):
    case, tris = CASES[name]
    rec = GOLDEN[name]
    fws = case.fws.copy()
    minus, plus = port.ibm(case, fws, tris)
    assert len(minus[0]) == rec["minus_count"] and len(plus[0]) == rec["plus_count"]
    assert _sha(ibm_files.text(*minus).encode()) == rec["minus"]
    assert _sha(ibm_files.text(*plus).encode()) == rec["plus"]
    assert hashlib.sha256(canonical(fws)).hexdigest() == rec["fws"]
    assert int((fws != case.fws).sum()) == rec["fws_changed"]


def test_fixture_cases_cover_every_branch(port):
    """Across the fixture cases: entries in both tables and ghost cells
    turned fluid.  (They also hold ghost cells without any ray hit, which
    take the closest-point fallback: 24, 24 and 59 of 200 in sphere_n8_l1,
    sphere_n8_l5 and sphere_n8_l2_offset.)"""
    seen = dict(minus=0, plus=0, fluid=0)
    for name, (case, tris) in CASES.items():
        fws = case.fws.copy()
        minus, plus = port.ibm(case, fws, tris)
        seen["minus"] += len(minus[0])
        seen["plus"] += len(plus[0])
        seen["fluid"] += int((fws != case.fws).sum())
    assert all(v > 0 for v in seen.values()), seen


def test_weights_interpolate_the_image_point(port):
    """Each entry's eight weights sum to 1 and reproduce the image point's
    position from the base cell's corners (trilinear interpolation of x, y
    and z is exact)."""
    case, tris = CASES["sphere_n8_l5"]
    fws = case.fws.copy()
    n = case.n
    for gc, ip, w in port.ibm(case, fws, tris):
        for g, p, ww in zip(gc, ip, w):
            c = p[0]
            dx = case.cube_size[c] / n
            base = case.origin[c] + (np.array(p[1:4]) - 1.5) * dx
            corners = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 0], [1, 0, 1],
                                [0, 1, 1], [1, 1, 1]], np.float64)
            pos = (ww[:, None] * (base + corners * dx)).sum(axis=0)
            centre = case.origin[g[0]] + (np.array(g[1:4]) - 1.5) * dx
            # the image point lies within sqrt(2) cells of twice the distance
            assert np.linalg.norm(pos - centre) <= 2 * np.sqrt(2) * dx + 1e-9
            assert abs(ww.sum() - 1.0) < 1e-9


def test_stl_round_trip(tmp_path):
    tris = cases.icosphere(2, 0.5, center=(0.1, 0.2, -0.3))
    path = str(tmp_path / "BCM_STL_fine.stl")
    cases.write_stl(path, tris)
    assert np.array_equal(cases.read_stl(path), tris)
    nrm = np.cross(tris[:, 1] - tris[:, 0], tris[:, 2] - tris[:, 0])
    out = (tris.mean(axis=1) - np.array([0.1, 0.2, -0.3]))
    assert (np.einsum("ij,ij->i", nrm, out) > 0).all()  # outward normals


def test_table_files_round_trip(tmp_path, port):
    case, tris = CASES["sphere_n8_l2_offset"]
    minus, _ = port.ibm(case, case.fws.copy(), tris)
    path = tmp_path / "IBM_minus00000.dat"
    path.write_text(ibm_files.text(*minus))
    gc, ip, w = ibm_files.read(str(path))
    assert np.array_equal(gc, minus[0]) and np.array_equal(ip, minus[1])
    assert np.allclose(w, minus[2], atol=5e-7)


@pytest.mark.skipif(not O.reference_available(), reason="reference sources not present")
def test_restatement_equals_reference_directly(tmp_path, port):
    """A case outside the fixtures: shifted, smaller sphere, 320 triangles."""
    case, _ = CASES["sphere_n8_l1"]
    tris = cases.icosphere(2, 0.41, center=(-0.21, 0.11, 0.02))
    cases.write_stl(str(tmp_path / "BCM_STL_fine.stl"), tris)
    fr, fo = case.fws.copy(), case.fws.copy()
    O.Ref(case).ibm(case, fr, str(tmp_path))
    minus, plus = port.ibm(case, fo, tris)
    assert np.array_equal(fr, fo)
    assert (tmp_path / "IBM_minus00000.dat").read_text() == ibm_files.text(*minus)
    assert (tmp_path / "IBM_plus00000.dat").read_text() == ibm_files.text(*plus)
