"""Build recipe for ``oracle/_ref``: the reference's own CPU code as a library.

TEST INFRASTRUCTURE ONLY.  This compiles the reference's C++ sources where they
lie (the directory named by ``BCM_REFERENCE_DIR``, by default ``reference``
beside this repository's root; read-only, nothing is copied) into
``oracle/_ref/libbcmref_<config>.so`` together with ``oracle/ref_driver.cpp``
(which only forwards arrays and replays the reference's per-stage call order).

The reference fixes its resolution and physical constants at compile time in
``Resolution.h`` and ``prm.h``, which every routine includes by a quoted
``#include``.  Quoted includes normally resolve next to the including file
first, so a per-configuration header cannot shadow the reference's own through
``-I``.  GCC's ``-I-`` switch turns that lookup off: directories given before
``-I-`` are searched first for quoted includes and the including file's own
directory is not searched.  The generated headers go to
``oracle/_ref/cfg_<config>/`` and keep the reference's macro names and
(unparenthesised) macro bodies, because the reference's expressions depend on
them textually (``Resolution.h:1-32``, ``prm.h:1-43``).

Build flags: ``-O2 -fopenmp -ffp-contract=off``.  ``-ffp-contract=off`` matters
on aarch64, where GCC otherwise fuses multiply-adds and the results stop being
the IEEE sequence the reference's source spells out.

When the reference directory is absent (the GPU host), nothing is built and the
tests that need the compiled reference skip; the committed golden fixtures in
``tests/golden`` carry its outputs instead.
"""
from __future__ import annotations

import os
import subprocess
import sys
from dataclasses import dataclass, field

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.environ.get("BCM_REFERENCE_DIR",
                         os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
OUT_DIR = os.path.join(HERE, "_ref")

# The reference translation units on the hot path.
REF_SOURCES = [
    "BCM_Flux_XYZ_Viscous_Runge_kutta.cpp",
    "BCM_Interface.cpp",
    "BCM_Interface_table.cpp",
    "BCM_Ghostcell_minus.cpp",
    "BCM_Ghostcell_plus.cpp",
    "BCM_X_boundary_condition.cpp",
    "BCM_Y_boundary_condition.cpp",
    "BCM_Z_boundary_condition.cpp",
    "BCM_Output.cpp",
    "BCM_Immersed_boundary.cpp",
    "BCM_FWS_Interface.cpp",
]


@dataclass(frozen=True)
class RefConfig:
    """Compile-time configuration of one reference build.

    ``ncube_x`` is the interior cells per cube edge (``NcubeX``), ``mpi_ncube``
    the global cube count used by the residual-norm normaliser
    (``BCM_Flux_XYZ_Viscous_Runge_kutta.cpp:2628``) and ``rank_map`` size.
    The physical constants are the ``prm.h`` doubles.
    """

    name: str
    ncube_x: int = 16
    mpi_ncube: int = 64
    mu_L: float = 0.0000185
    rho0: float = 1.1842
    U0: float = 38.889
    Uin: float = 38.889
    P0: float = 101300.0
    extra: dict = field(default_factory=dict, compare=False, hash=False)


def _fmt(x: float) -> str:
    return repr(float(x))


def resolution_h(c: RefConfig) -> str:
    n = c.ncube_x
    # Same macro names and textual bodies as the reference's Resolution.h.
    return "\n".join([
        "#define np 1",
        f"#define MPI_Ncube {c.mpi_ncube}",
        "#define n_buffer 2",
        f"#define NcubeX {n}",
        f"#define NcubeY {n}",
        f"#define NcubeZ {n}",
        "#define Ndim 5",
        "#define nx NcubeX + n_buffer - 1",
        "#define ny NcubeY + n_buffer - 1",
        "#define nz NcubeZ + n_buffer - 1",
        f"#define X_size {n + 4}",
        f"#define Y_size {n + 4}",
        f"#define Z_size {n + 4}",
        "#define nxx nx+1",
        "#define nyy ny+1",
        "#define nzz nz+1",
        "#define nxxx nxx+1",
        "#define nyyy nyy+1",
        "#define nzzz nzz+1",
        "",
    ])


def prm_h(c: RefConfig) -> str:
    # Same names as the reference's prm.h; K and R keep their literal spelling
    # because the reference's arithmetic uses the macro text (e.g. (K-1)).
    return "\n".join([
        "#define K 1.4",
        "#define R 287",
        "#define Cv 717.5",
        f"#define mu_L {_fmt(c.mu_L)}",
        "#define Pr_L 0.72",
        "double Cp = Cv*K;",
        "double lambda_L = mu_L*Cv*K/Pr_L;",
        "#define Ep 1.",
        "#define MAX 100000000",
        "#define MIN -100000000",
        "#define minimum 0.0000001",
        "double psi = 0.0001;",
        f"double rho0 = {_fmt(c.rho0)};",
        f"double U0 = {_fmt(c.U0)};",
        f"double Uin = {_fmt(c.Uin)};",
        "double V0 = 0.;",
        "double W0 = 0;",
        f"double P0 = {_fmt(c.P0)};",
        "double T0 = P0/rho0/R;",
        "",
    ])


def reference_available() -> bool:
    return all(os.path.isfile(os.path.join(REF_DIR, s)) for s in REF_SOURCES)


def lib_path(c: RefConfig) -> str:
    return os.path.join(OUT_DIR, f"libbcmref_{c.name}.so")


def build(c: RefConfig, force: bool = False, verbose: bool = False) -> str | None:
    """Compile the reference for configuration ``c``; returns the .so path.

    Returns None when the reference sources are not present on this machine.
    """
    out = lib_path(c)
    cfg_dir = os.path.join(OUT_DIR, f"cfg_{c.name}")
    if not reference_available():
        return out if os.path.isfile(out) else None
    os.makedirs(cfg_dir, exist_ok=True)
    want = {"Resolution.h": resolution_h(c), "prm.h": prm_h(c)}
    changed = False
    for fn, text in want.items():
        p = os.path.join(cfg_dir, fn)
        if not os.path.isfile(p) or open(p).read() != text:
            with open(p, "w") as f:
                f.write(text)
            changed = True
    driver = os.path.join(HERE, "ref_driver.cpp")
    recipe = [driver, os.path.abspath(__file__), os.path.join(HERE, "mpi_stub", "mpi.h")]
    if os.path.isfile(out) and not (force or changed):
        if os.path.getmtime(out) >= max(os.path.getmtime(x) for x in recipe):
            return out
    srcs = [os.path.join(REF_DIR, s) for s in REF_SOURCES] + [driver]
    cmd = [
        # C++14: the reference is C++98-style code, and a C++17 <algorithm>
        # pulls in parallel-STL headers whose quoted includes -I- would hide
        "g++", "-std=gnu++14", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-w",
        "-I", cfg_dir, "-I-", "-I", os.path.join(HERE, "mpi_stub"), "-I", REF_DIR,
        *srcs, "-o", out + ".tmp",
    ]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed for {c.name}:\n{r.stderr[-4000:]}")
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build(RefConfig("default16"), force=True, verbose=True))
