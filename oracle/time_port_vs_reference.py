"""How fast the C restatement runs against the reference's own compiled code.

TEST INFRASTRUCTURE ONLY.  The benchmark's CPU baseline and reference arm
time the C restatement (oracle/bcm_oracle.c) because the reference's sources
are not on the GPU host and its build here does not run there.  This script
times both on a host where the reference compiles (oracle/ref_build.py,
BCM_REFERENCE_DIR): one dual-time step of two sub-iterations of the same
case, same OpenMP thread count, after one untimed step, and prints
cell-sub-iterations per second and the ratio.

    python oracle/time_port_vs_reference.py
"""
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.dirname(HERE), HERE]

import oracle as O  # noqa: E402
from bcm_cgli_gb300 import cases  # noqa: E402


def main():
    for name, case in (("vortex 4^3 cubes of 16^3", cases.isentropic_vortex(ncx=4, n=16)),
                       ("taylor-green 4^3 cubes of 24^3", cases.taylor_green(ncx=4, n=24))):
        for threads in (1, os.cpu_count() or 1):
            rate = {}
            for kind, runner in (("reference", O.Ref(case)), ("port", O.Port())):
                runner.set_threads(threads)
                runner.run(case, O.State(case), 1, 1)
                st = O.State(case)
                t0 = time.perf_counter()
                runner.run(case, st, 1, 2)
                rate[kind] = case.n_cells * 2 / (time.perf_counter() - t0)
            print(f"{name}, {threads} threads: reference {rate['reference']:.3e}, "
                  f"restatement {rate['port']:.3e} cell-subiters/s, "
                  f"ratio {rate['port'] / rate['reference']:.2f}", flush=True)


if __name__ == "__main__":
    main()
