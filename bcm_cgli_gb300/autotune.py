"""Launch-shape autotuner: times the candidate shapes of the hot kernels on
this GPU and writes the table the benchmark applies.

    python -m bcm_cgli_gb300.autotune [--out bcm_cgli_gb300/tuning_gb300.json]

For every cube resolution n of the benchmark workloads (16, 24, 32) and each
path (FP64 / split precision, RK / LU-SGS sub-iterations) it builds a
Taylor-Green case of 2-3 million cells (8^3 cubes of 16^3, 6^3 of 24^3, 4^3
of 32^3: many waves of CTAs, as in the benchmark workloads; a case of a
wave or two favours the smaller tile through its tail alone), lets
bcmg_case_autotune time the flux tile edges (8, 4) and, for split LU-SGS,
the sweep's thread counts (widest plane, half of it), and records the
fastest shape with the measured times.  The shapes change how work is
spread over the GPU, never a cell's arithmetic.
"""
from __future__ import annotations

import argparse
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_TABLE = os.path.join(HERE, "tuning_gb300.json")


def key(n: int, precision: str, method: str) -> str:
    return f"n{n}_{precision}_{method}"


def lookup(n: int, precision: str, method: str, path: str = DEFAULT_TABLE):
    """The stored shape for (n, precision, method), or None."""
    try:
        with open(path) as f:
            return json.load(f)["shapes"].get(key(n, precision, method))
    except (OSError, ValueError, KeyError):
        return None


def tune(reps: int = 3):
    from . import api, cases
    shapes = {}
    for n, ncx in ((16, 8), (24, 6), (32, 4)):
        case = cases.taylor_green(ncx=ncx, n=n)
        for precision in ("fp64", "split"):
            for method in ("rk3", "lusgs"):
                prec = api.PRECISION_SPLIT if precision == "split" else api.PRECISION_FP64
                ctx = api.CaseContext(case, precision=prec)
                if method == "lusgs":
                    ctx.set_method(api.METHOD_LUSGS)
                ctx.set_state(case.U, case.U, case.U)
                res = ctx.autotune(reps)
                ctx.close()
                res["case"] = f"taylor_green(ncx={ncx}, n={n})"
                shapes[key(n, precision, method)] = res
                print(key(n, precision, method), res, flush=True)
    return shapes


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_TABLE)
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args()
    shapes = tune(args.reps)
    import torch  # noqa: F401  (device name only)
    name = torch.cuda.get_device_name(0) if torch.cuda.is_available() else "unknown"
    with open(args.out, "w") as f:
        json.dump({"device": name, "generator": "python -m bcm_cgli_gb300.autotune",
                   "shapes": shapes}, f, indent=1)


if __name__ == "__main__":
    main()
