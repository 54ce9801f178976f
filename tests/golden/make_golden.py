"""Generate tests/golden/golden.json from the REFERENCE's own compiled code.

Runs each case of golden_cases.py through oracle/_ref (the reference's
BCM_*.cpp compiled where they lie (BCM_REFERENCE_DIR) by oracle/ref_build.py, one OpenMP
thread so its norm sums are serial) and records SHA-256 digests of every
output array plus the norms.  Run here, where the reference sources exist:

    python tests/golden/make_golden.py            # everything
    python tests/golden/make_golden.py --ibm-only # the IBM preprocessing records
    python tests/golden/make_golden.py --horizon  # the long-run records only
    python tests/golden/make_golden.py --flags    # the flag-interface records only
"""
import hashlib
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), HERE]

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402
from golden_cases import (RUN_STEPS, RUN_SUBITERS, canonical, flag_cases,  # noqa: E402
                          golden_cases, horizon_cases, ibm_cases)
from bcm_cgli_gb300 import cases as _cases  # noqa: E402


def digest(a):
    return hashlib.sha256(canonical(a)).hexdigest()


def ibm_records():
    """Digests of the reference's BCM_Immersed_boundary outputs: the two
    table files (text) and the flags after it."""
    out = {}
    for name, (case, tris) in ibm_cases().items():
        fws = case.fws.copy()
        with tempfile.TemporaryDirectory() as d:
            _cases.write_stl(os.path.join(d, "BCM_STL_fine.stl"), tris)
            O.Ref(case).ibm(case, fws, d)
            rec = {"fws": digest(fws), "fws_changed": int((fws != case.fws).sum())}
            for side in ("minus", "plus"):
                with open(os.path.join(d, f"IBM_{side}00000.dat"), "rb") as f:
                    txt = f.read()
                rec[side] = hashlib.sha256(txt).hexdigest()
                rec[side + "_count"] = int(txt.rsplit(b"\n", 1)[-1])
        out[name] = rec
        print(name, "done", file=sys.stderr)
    return out


def horizon_records():
    """Digests of the state after the long runs of horizon_cases(): the
    reference's own loop (one OpenMP thread) over every dual-time step and
    sub-iteration of the configuration."""
    out = {}
    for name, (case, steps, subiters) in horizon_cases().items():
        ref = O.Ref(case)
        ref.set_threads(1)
        st = O.State(case)
        ref.run(case, st, steps, subiters)
        out[name] = {"steps": steps, "subiters": subiters, "initial": digest(case.U),
                     "state": {k: digest(getattr(st, k)) for k in ("U1_", "U1", "U1q")},
                     "er": [repr(float(x)) for x in st.er],
                     "sum": [repr(float(x)) for x in st.U1_.reshape(-1, 5).sum(axis=0)]}
        print(name, "done", file=sys.stderr)
    return out


def flag_records():
    """Digests of the flags after the reference's BCM_FWS_Interface on one
    rank (its own same-level lists), the input flags' digest, and how many
    flags it changed."""
    out = {}
    for name, case in flag_cases().items():
        fws = case.fws.copy()
        O.Ref(case).fws_interface(case, fws)
        out[name] = {"input": digest(case.fws), "fws": digest(fws),
                     "changed": int((fws != case.fws).sum())}
        print(name, "done", file=sys.stderr)
    return out


def main():
    path = os.path.join(HERE, "golden.json")
    if "--horizon" in sys.argv:
        with open(path) as f:
            doc = json.load(f)
        doc["horizon"] = horizon_records()
        with open(path, "w") as f:
            json.dump(doc, f, indent=1)
        return
    if "--flags" in sys.argv:
        with open(path) as f:
            doc = json.load(f)
        doc["flags"] = flag_records()
        with open(path, "w") as f:
            json.dump(doc, f, indent=1)
        return
    if "--ibm-only" in sys.argv:
        with open(path) as f:
            doc = json.load(f)
        doc["ibm"] = ibm_records()
        with open(path, "w") as f:
            json.dump(doc, f, indent=1)
        return
    out = {}
    for name, case in golden_cases().items():
        ref = O.Ref(case)
        ref.set_threads(1)
        rec = {}
        # single routines on the initial state
        for r, fn in (("bc", lambda s: ref.bc(case, s.U1_)),
                      ("ghost_minus", lambda s: ref.ghost(case, s.U1_, -1)),
                      ("ghost_plus", lambda s: ref.ghost(case, s.U1_, 1)),
                      ("interface", lambda s: ref.interface(case, s.U1_))):
            st = O.State(case)
            fn(st)
            rec[r] = digest(st.U1_)
        # three flux stages on the initial state
        st = O.State(case)
        for RK in (1, 2, 3):
            ref.flux_stage(case, st, RK)
            rec[f"flux{RK}"] = {k: digest(getattr(st, k))
                                for k in ("U1_", "Rku1", "Residual1", "U1p1", "U1p2")}
        rec["flux3_er"] = [repr(float(x)) for x in st.er]
        # full loop
        st = O.State(case)
        ref.run(case, st, RUN_STEPS, RUN_SUBITERS)
        rec["run"] = {k: digest(getattr(st, k)) for k in ("U1_", "U1", "U1q", "Rku1",
                                                          "Residual1")}
        rec["run_er"] = [repr(float(x)) for x in st.er]
        rec["run_emax"] = [repr(float(x)) for x in st.Emax]
        rec["run_sum"] = [repr(float(x)) for x in st.U1_.reshape(-1, 5).sum(axis=0)]
        # the reference's PLOT3D writer (BCM_Output.cpp) on the final state
        with tempfile.TemporaryDirectory() as d:
            ref.output(case, st.U1_, 7, d)
            for key, fn in (("plot3d_x", "BCMdata00001.x"), ("plot3d_q", "qBCMdata00007.q")):
                with open(os.path.join(d, fn), "rb") as f:
                    rec[key] = hashlib.sha256(f.read()).hexdigest()
        out[name] = rec
        print(name, "done", file=sys.stderr)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py (reference compiled by "
                                "oracle/ref_build.py, OMP_NUM_THREADS=1)",
                   "steps": RUN_STEPS, "subiters": RUN_SUBITERS, "cases": out,
                   "ibm": ibm_records(), "horizon": horizon_records(),
                   "flags": flag_records()}, f, indent=1)


if __name__ == "__main__":
    main()
