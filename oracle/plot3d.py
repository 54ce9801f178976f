"""ORACLE (test infrastructure): PLOT3D output as BCM_Output writes it.

Restates the file layout of BCM_Output.cpp:16-300 (one rank), used to check
the GPU writer byte for byte; the restatement itself is pinned against the
reference's compiled BCM_Output (tests/test_plot3d.py) where the reference
sources are present.

Both files are raw (no Fortran record markers), native endian:
  header: int32 MPI_Ncube, then (n+2, n+2, n+2) as int32 for each of the
          MPI_Ncube cubes (:101-120, :204-218);
  grid  (BCMdata00001.x): per cube 1..ncube-1 three blocks of (n+2)^3
          doubles, X then Y then Z, over padded indices 1..n+2 with the
          first array index fastest (:127-166); cell centres
          Xcube + (i - 1.5) dx (BCM_Grid.cpp:124-148);
  solution (qBCMdata<step>.q): per cube four 1.0 doubles, then the five
          conservative variables, each an (n+2)^3 block in the same order
          (:222-291), of the current state U1_ (main.cpp:1348).
"""
from __future__ import annotations

import numpy as np


def header(n: int, ncube_out: int) -> bytes:
    h = np.empty(1 + 3 * ncube_out, np.int32)
    h[0] = ncube_out
    h[1:] = n + 2
    return h.tobytes()


def grid_bytes(n: int, ncube: int, cube_size, origin, ncube_out: int) -> bytes:
    m = n + 2
    idx = np.arange(1, n + 3, dtype=np.float64)
    parts = [header(n, ncube_out)]
    for c in range(1, ncube):
        dx = cube_size[c] / n
        X = origin[c, 0] + (idx - 1.5) * dx
        Y = origin[c, 1] + (idx - 1.5) * dx
        Z = origin[c, 2] + (idx - 1.5) * dx
        parts.append(np.broadcast_to(X[None, None, :], (m, m, m)).tobytes())
        parts.append(np.broadcast_to(Y[None, :, None], (m, m, m)).tobytes())
        parts.append(np.broadcast_to(Z[:, None, None], (m, m, m)).tobytes())
    return b"".join(parts)


def solution_bytes(n: int, U: np.ndarray, ncube_out: int) -> bytes:
    parts = [header(n, ncube_out)]
    ones = np.ones(4).tobytes()
    for c in range(1, U.shape[0]):
        parts.append(ones)
        sub = U[c, 1:n + 3, 1:n + 3, 1:n + 3, :]  # [x][y][z][v]
        for v in range(5):
            parts.append(np.ascontiguousarray(sub[:, :, :, v].transpose(2, 1, 0)).tobytes())
    return b"".join(parts)
