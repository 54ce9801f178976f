"""The one-pass forms of the edge fill and the boundary fill, on the CPU.

The reference fills ghost cells in ordered phases: the edge fill as i-edges,
then j-edges and k-edges over the whole ghost range
(BCM_Interface.cpp:5640-5732); the boundary fill as x faces, then y faces
over every i, then z faces over every i, j (BCM_X/Y/Z_boundary_condition.cpp,
main.cpp:1161-1165).  The kernels `k_iface_edges` and `k_bc` form every
written cell in one pass from cells no phase writes.  These tests state both
rules in numpy and require them to leave every cell as the ordered phases do,
bit for bit, on random states (every boundary mask and axis subset for the
boundary fill).  The GPU parity tests compare the kernels themselves with the
oracle.
"""
import numpy as np
import pytest

K = 1.4


def _edges_phased(U, n):
    U = U.copy()
    nx, nyy = n + 1, n + 2

    def avg(d, x, y):
        U[d] = 0.5 * (U[x] + U[y])
    for i in range(2, nx + 1):
        avg((i, 1, 1), (i, 1, 2), (i, 2, 1))
        avg((i, nyy, 1), (i, nyy, 2), (i, nx, 1))
        avg((i, 1, nyy), (i, 1, nx), (i, 2, nyy))
        avg((i, nyy, nyy), (i, nyy, nx), (i, nx, nyy))
    for j in range(1, nyy + 1):
        avg((1, j, 1), (1, j, 2), (2, j, 1))
        avg((1, j, nyy), (2, j, nyy), (1, j, nx))
        avg((nyy, j, 1), (nx, j, 1), (nyy, j, 2))
        avg((nyy, j, nyy), (nx, j, nyy), (nyy, j, nx))
    for k in range(1, nyy + 1):
        avg((1, 1, k), (1, 2, k), (2, 1, k))
        avg((1, nyy, k), (2, nyy, k), (1, nx, k))
        avg((nyy, 1, k), (nx, 1, k), (nyy, 2, k))
        avg((nyy, nyy, k), (nx, nyy, k), (nyy, nx, k))
    return U


def _edges_one_pass(U, n):
    out = U.copy()
    nx, nyy = n + 1, n + 2

    def inward(x):
        return 2 if x == 1 else nx

    def edge(c):  # two ghost coordinates: average of the two inward face ghosts
        a, b = [t for t in range(3) if c[t] in (1, nyy)]
        p, q = list(c), list(c)
        p[a], q[b] = inward(p[a]), inward(q[b])
        return 0.5 * (U[tuple(p)] + U[tuple(q)])
    for free in range(3):
        others = [t for t in range(3) if t != free]
        for g1 in (1, nyy):
            for g2 in (1, nyy):
                for pos in range(2, nx + 1):
                    c = [0, 0, 0]
                    c[free], c[others[0]], c[others[1]] = pos, g1, g2
                    out[tuple(c)] = edge(c)
    for i in (1, nyy):
        for j in (1, nyy):
            for k in (1, nyy):  # corner: the k-edge phase's j-edge and i-edge average
                out[i, j, k] = 0.5 * (edge((i, inward(j), k)) + edge((inward(i), j, k)))
    return out


def _inflow(q, Uin):
    rho = q[0]
    U0, V0, W0 = q[1] / rho, q[2] / rho, q[3] / rho
    VV = U0 * U0 + V0 * V0 + W0 * W0
    P = (q[4] - 0.5 * rho * VV) * (K - 1)
    Uu, Vv, Ww = Uin, 0.0, 0.0
    VV = Uu * Uu + Vv * Vv + Ww * Ww
    return np.array([rho, rho * Uu, rho * Vv, rho * Ww, P / (K - 1) + 0.5 * rho * VV])


def _bc_phased(Q, n, m, axes, Uin):
    Q = Q.copy()
    S, nx, nxx, nxxx = n + 4, n + 1, n + 2, n + 3
    interior = range(2, n + 2)
    if axes & 1:
        for j in interior:
            for k in interior:
                if m & 1:
                    Q[0, j, k] = Q[1, j, k] = _inflow(Q[2, j, k], Uin)
                if m & 2:
                    Q[nxx, j, k] = Q[nxxx, j, k] = Q[nx, j, k]
    if axes & 2:
        for i in range(S):
            for k in interior:
                if m & 4:
                    Q[i, 0, k] = Q[i, 1, k] = Q[i, 2, k]
                if m & 8:
                    Q[i, nxx, k] = Q[i, nxxx, k] = Q[i, nx, k]
    if axes & 4:
        for i in range(S):
            for j in range(S):
                if m & 16:
                    x = Q[i, j, 2].copy()
                    x[3] = -x[3]
                    Q[i, j, 0] = Q[i, j, 1] = x
                if m & 32:
                    Q[i, j, nxx] = Q[i, j, nxxx] = Q[i, j, nx]
    return Q


def _bc_one_pass(Q0, n, m, axes, Uin):
    Q = Q0.copy()
    S, nx, nxx, nxxx = n + 4, n + 1, n + 2, n + 3
    mx = m & 3 if axes & 1 else 0
    my = (m >> 2) & 3 if axes & 2 else 0
    mz = (m >> 4) & 3 if axes & 4 else 0

    def interior(x):
        return 2 <= x <= nx

    def read(i, j, k, upto):  # the cell as the ordered phases leave it, from unwritten cells
        if upto >= 2 and my and interior(k):
            if (my & 1) and j <= 1:
                j = 2
            elif (my & 2) and j >= nxx:
                j = nx
        if mx and interior(j) and interior(k):
            if (mx & 1) and i <= 1:
                return _inflow(Q0[2, j, k], Uin)
            if (mx & 2) and i >= nxx:
                i = nx
        return Q0[i, j, k].copy()
    for j in range(2, n + 2):
        for k in range(2, n + 2):
            if mx & 1:
                Q[0, j, k] = Q[1, j, k] = _inflow(Q0[2, j, k], Uin)
            if mx & 2:
                Q[nxx, j, k] = Q[nxxx, j, k] = Q0[nx, j, k]
    for i in range(S):
        for k in range(2, n + 2):
            if my & 1:
                Q[i, 0, k] = Q[i, 1, k] = read(i, 2, k, 1)
            if my & 2:
                Q[i, nxx, k] = Q[i, nxxx, k] = read(i, nx, k, 1)
    for i in range(S):
        for j in range(S):
            if mz & 1:
                x = read(i, j, 2, 2)
                x[3] = -x[3]
                Q[i, j, 0] = Q[i, j, 1] = x
            if mz & 2:
                Q[i, j, nxx] = Q[i, j, nxxx] = read(i, j, nx, 2)
    return Q


@pytest.mark.parametrize("n", [4, 8, 16])
def test_edge_fill_in_one_pass(n):
    rng = np.random.default_rng(n)
    S = n + 4
    U = rng.standard_normal((S, S, S, 5)) * 10.0 ** rng.integers(-3, 4, (S, S, S, 1))
    a, b = _edges_phased(U, n), _edges_one_pass(U, n)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("n", [4, 8])
def test_boundary_fill_in_one_pass(n):
    rng = np.random.default_rng(7 + n)
    S = n + 4
    for m in range(64):
        for axes in (7, 1, 2, 4, 3, 6, 5):  # the context's call, and the per-axis twins
            Q = rng.standard_normal((S, S, S, 5))
            Q[..., 0] = 1 + rng.random((S, S, S))
            a, b = _bc_phased(Q, n, m, axes, 0.7), _bc_one_pass(Q, n, m, axes, 0.7)
            assert np.array_equal(a.view(np.uint64), b.view(np.uint64)), (m, axes)
