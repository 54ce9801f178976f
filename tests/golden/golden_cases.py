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


def horizon_cases():
    """(case, steps, sub-iterations) of the long-run records: the inviscid
    isentropic vortex of 4x4x4 cubes of 16^3 cells (262,144 cells, Mach 0.5,
    strength 5, dT = 1e-3) over its whole run of 100 dual-time steps x 10
    RK sub-iterations."""
    return {"vortex_full": (cases.isentropic_vortex(ncx=4, n=16, dT=1e-3), 100, 10)}


def flag_cases():
    """Cases for the flag-field interface fixtures (BCM_FWS_Interface):
    random flags with many solid cells, so that holes form and fill in
    chains; every cube on the finest level (csl = 0, the only level the
    routine changes) except in the two-level case, whose coarse cubes must
    keep their flags.  A one-cube periodic box makes a cube its own
    neighbour on every axis."""
    def finest(case):
        case.csl = np.zeros_like(case.csl)
        return case
    return {
        "flags_periodic_n8": finest(cases.random_case(seed=21, ncx=2, ncy=2, ncz=1, n=8,
                                                      periodic=True, solid_frac=0.35,
                                                      ghost_frac=0.2)),
        "flags_open_n4": finest(cases.random_case(seed=22, ncx=3, ncy=2, ncz=2, n=4,
                                                  periodic=False, solid_frac=0.4,
                                                  ghost_frac=0.2)),
        "flags_two_level_n4": cases.random_two_level_case(seed=23, n=4, periodic=True,
                                                          solid_frac=0.4, ghost_frac=0.2),
        "flags_one_cube_n4": finest(cases.random_case(seed=24, ncx=1, ncy=1, ncz=1, n=4,
                                                      periodic=True, solid_frac=0.45,
                                                      ghost_frac=0.2)),
    }


def ibm_cases():
    """(case, triangles) pairs for the IBM preprocessing fixtures: a sphere of
    diameter 1 on a two-level grid of n=8 cubes (fine cubes of edge 1, cells
    of 1/8), as icospheres of 80, 1,280 and 20,480 triangles.  The coarse
    80-triangle body and the off-centre sphere leave many ghost cells
    without any ray hit (closest-point fallback, carried side test)."""
    def grid():
        return cases.sphere_ibm(n=8, coarse=2.0, box=((-2.0, 4.0), (-2.0, 2.0), (-2.0, 2.0)),
                                refine_box=((-2.0, 2.0), (-2.0, 2.0), (-2.0, 2.0)))
    return {
        "sphere_n8_l1": (grid(), cases.icosphere(1, 0.5)),
        "sphere_n8_l3": (grid(), cases.icosphere(3, 0.5)),
        "sphere_n8_l5": (grid(), cases.icosphere(5, 0.5)),
        "sphere_n8_l2_offset": (grid(), cases.icosphere(2, 0.45, center=(0.13, -0.07, 0.05))),
    }
