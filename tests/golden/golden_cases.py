"""The small cases the golden fixtures are made from (shared by the
generator and the tests).  Sizes are chosen so the reference finishes each
in well under a second."""
import numpy as np

from bcm_cgli_gb300 import cases


def canonical(a: np.ndarray) -> bytes:
    """Bytes of an array with -0.0 folded to +0.0 (signed zeros are equal
    values and may differ between two correct evaluations)."""
    a = np.ascontiguousarray(a)
    if a.dtype.kind == "f":
        a = a + 0.0
    return a.tobytes()


def golden_cases():
    return {
        # open box, viscous, random flags and IBM tables: every branch
        "random_open_n4": cases.random_case(seed=11, n=4, periodic=False, viscous=True),
        # periodic, viscous, flags, IBM
        "random_periodic_n8": cases.random_case(seed=12, ncx=2, ncy=1, ncz=2, n=8,
                                                periodic=True, viscous=True),
        # inviscid isentropic vortex, 2x2x2 cubes of 8^3 (config-1 physics, small)
        "vortex_n8": cases.isentropic_vortex(ncx=2, n=8, dT=1e-3),
        # viscous Taylor-Green, 2x2x2 cubes of 8^3 (config-2 physics, small)
        "tgv_n8": cases.taylor_green(ncx=2, n=8),
        # two cube levels (one coarse cube refined 2:1), periodic and open:
        # every coarse<->fine interface block (config-3 structure, small)
        "two_level_periodic_n4": cases.random_two_level_case(seed=5, n=4, periodic=True,
                                                             solid_frac=0.03, ghost_frac=0.03),
        "two_level_open_n8": cases.random_two_level_case(seed=6, n=8, periodic=False),
    }


RUN_STEPS = 2
RUN_SUBITERS = 2
