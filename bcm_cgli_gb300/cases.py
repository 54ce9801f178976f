"""Synthetic BCM cases: cube grids, adjacency, flags, initial fields.

A *case* is everything the hot path consumes, in the reference's own layout
(``Array.h:13-44``): conservative state ``U[c][i][j][k][5]`` with ``S = n+4``
cells per cube edge (two ghost layers each side), flags ``FWS[c][i][j][k]``,
``cube_size[c]``, level ``csl[c]`` and adjacency ``adj_number[c][5][7]``
(slot 1..4, direction 1..6 = -x,+x,-y,+y,-z,+z; ``BCM_Grid.cpp`` layout).
Cube 0 is unused: the reference numbers cubes from 1 (``main.cpp:90``).

All random inputs come from a counter-based generator (splitmix64 on the
cell index) so fixtures are identical on every machine and numpy version.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

GAMMA = 1.4  # K, prm.h:1
R_GAS = 287.0  # R, prm.h:2
CV = 717.5  # Cv, prm.h:4
PR_L = 0.72  # Pr_L, prm.h:6

IFLUID, IGHOST, ISOLID = 1, 0, -1  # BCM.h:6-8


def splitmix_uniform(seed: int, count: int) -> np.ndarray:
    """Deterministic uniforms in [0,1) from splitmix64(seed*2^32 + index)."""
    with np.errstate(over="ignore"):
        x = (np.arange(count, dtype=np.uint64) + np.uint64(seed) * np.uint64(1 << 32))
        x = x + np.uint64(0x9E3779B97F4A7C15)
        z = x.copy()
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


@dataclass
class Phys:
    """prm.h constants of one case (plus the MPI_Ncube norm normaliser)."""

    mu_L: float = 0.0000185
    rho0: float = 1.1842
    U0: float = 38.889
    Uin: float = 38.889
    P0: float = 101300.0
    mpi_ncube: int = 64

    @property
    def T0(self) -> float:
        return self.P0 / self.rho0 / R_GAS


@dataclass
class Case:
    n: int  # interior cells per cube edge (NcubeX)
    ncube: int  # number of cube slots incl. the unused slot 0 (reference Ncube)
    phys: Phys
    cube_size: np.ndarray  # [ncube] f64
    csl: np.ndarray  # [ncube] i32
    origin: np.ndarray  # [ncube, 3] f64 (Xcube, Ycube, Zcube)
    adj: np.ndarray  # [ncube, 5, 7] i32
    fws: np.ndarray  # [ncube, S, S, S] i32
    U: np.ndarray  # [ncube, S, S, S, 5] f64 initial state (all cells)
    dT: float = 1e-4
    dTau: float = 1e-4 / 200.0
    e: float = 0.1
    name: str = "case"
    # IBM ghost tables, 1-based packed like BCM_Reading_IBM.cpp:53-73.
    ibm_minus: tuple | None = None  # (weight[8n+1], GCindex[4n+1], IPsur[4n+1])
    ibm_plus: tuple | None = None
    meta: dict = field(default_factory=dict)
    # Boundary-cube lists given explicitly (a rank's share of a sharded case,
    # whose own bounding box is not the domain's); None: from the geometry.
    bc: tuple | None = None

    @property
    def S(self) -> int:
        return self.n + 4

    @property
    def n_cells(self) -> int:
        """Interior cells of all real cubes (the unit of the throughput metric)."""
        return (self.ncube - 1) * self.n ** 3

    def bc_lists(self):
        """Boundary-cube lists by bounding box, as main.cpp:108-189 builds them.

        Returns six int32 arrays (x lower, x upper, y lower, y upper, z lower,
        z upper) of cube numbers in increasing order.
        """
        if self.bc is not None:
            return [np.asarray(x, np.int32) for x in self.bc]
        c = np.arange(1, self.ncube)
        o = self.origin[1:]
        s = self.cube_size[1:]
        lo = [o[:, a].min() for a in range(3)]
        hi = [(o[:, a] + s).max() for a in range(3)]
        out = []
        for a in range(3):
            out.append(c[np.abs(o[:, a] - lo[a]) < 1e-7].astype(np.int32))
            out.append(c[np.abs(o[:, a] + s - hi[a]) < 1e-7].astype(np.int32))
        return out  # xl, xu, yl, yu, zl, zu

    def cell_centres(self):
        """Cell-centre coordinates [ncube, S] per axis: origin + (i-1.5)*dx
        (BCM_Grid.cpp: Xcnt = Xcube + (i-1.5)*dx)."""
        dx = self.cube_size / self.n
        idx = np.arange(self.S, dtype=np.float64) - 1.5
        return [self.origin[:, a][:, None] + idx[None, :] * dx[:, None] for a in range(3)]


def periodic_box(ncx: int, ncy: int, ncz: int, n: int, length: float):
    """Equal cubes tiling [0,L)^3 with wrap-around adjacency (slot 1 only).

    Cube numbering is x-fastest from 1.  Returns (ncube, cube_size, csl,
    origin, adj).  Periodicity comes only from the adjacency, like the
    reference (which has no periodic boundary condition).
    """
    nc = ncx * ncy * ncz
    ncube = nc + 1
    size = length / ncx
    cube_size = np.zeros(ncube)
    cube_size[1:] = size
    csl = np.zeros(ncube, np.int32)
    csl[1:] = 1
    origin = np.zeros((ncube, 3))
    adj = np.zeros((ncube, 5, 7), np.int32)
    def num(a, b, c):
        return 1 + (a % ncx) + ncx * ((b % ncy) + ncy * (c % ncz))
    for c in range(ncz):
        for b in range(ncy):
            for a in range(ncx):
                k = num(a, b, c)
                origin[k] = (a * size, b * size, c * size)
                adj[k, 1, 1] = num(a - 1, b, c)
                adj[k, 1, 2] = num(a + 1, b, c)
                adj[k, 1, 3] = num(a, b - 1, c)
                adj[k, 1, 4] = num(a, b + 1, c)
                adj[k, 1, 5] = num(a, b, c - 1)
                adj[k, 1, 6] = num(a, b, c + 1)
    return ncube, cube_size, csl, origin, adj


def open_box(ncx: int, ncy: int, ncz: int, n: int, length: float):
    """Like periodic_box but without wrap-around: domain faces have no
    neighbour, so the X/Y/Z boundary conditions stay visible."""
    ncube, cube_size, csl, origin, adj = periodic_box(ncx, ncy, ncz, n, length)
    for k in range(1, ncube):
        a = int(round(origin[k, 0] / cube_size[k]))
        b = int(round(origin[k, 1] / cube_size[k]))
        c = int(round(origin[k, 2] / cube_size[k]))
        if a == 0: adj[k, 1, 1] = 0
        if a == ncx - 1: adj[k, 1, 2] = 0
        if b == 0: adj[k, 1, 3] = 0
        if b == ncy - 1: adj[k, 1, 4] = 0
        if c == 0: adj[k, 1, 5] = 0
        if c == ncz - 1: adj[k, 1, 6] = 0
    return ncube, cube_size, csl, origin, adj


def conservative(rho, u, v, w, p):
    """(rho, rho u, rho v, rho w, E) with E = p/(K-1) + rho|u|^2/2."""
    E = p / (GAMMA - 1) + 0.5 * rho * (u * u + v * v + w * w)
    return np.stack([rho, rho * u, rho * v, rho * w, E], axis=-1)


def _grid(case_geom, n):
    ncube, cube_size, csl, origin, adj = case_geom
    S = n + 4
    dx = cube_size / n
    idx = np.arange(S, dtype=np.float64) - 1.5
    X = origin[:, 0][:, None, None, None] + idx[None, :, None, None] * dx[:, None, None, None]
    Y = origin[:, 1][:, None, None, None] + idx[None, None, :, None] * dx[:, None, None, None]
    Z = origin[:, 2][:, None, None, None] + idx[None, None, None, :] * dx[:, None, None, None]
    X, Y, Z = np.broadcast_arrays(X, Y, Z)
    return X, Y, Z


def exp_portable(x):
    """exp(x) from IEEE additions, multiplications and exact scalings only,
    so the same inputs give the same bits on every machine (numpy's exp and
    pow differ in the last bit between x86 and Arm builds).  x = k ln2 + r
    with |r| <= ln2/2 (ln2 split in a 32-bit head and its tail, so k ln2 is
    exact), exp(r) by its Taylor series to r^16 in Horner form (truncation
    below 1e-17 relative), times 2^k."""
    x = np.asarray(x, dtype=np.float64)
    ln2_hi = 0.693145751953125          # 22 significant bits: k * ln2_hi is exact
    ln2_lo = 1.4286068203094172321e-06  # ln2 - ln2_hi
    k = np.floor(x / 0.6931471805599453 + 0.5)
    r = (x - k * ln2_hi) - k * ln2_lo
    p = np.ones_like(r)
    for m in range(16, 0, -1):
        p = 1.0 + r * p / m
    return np.ldexp(p, k.astype(np.int64))


def isentropic_vortex(ncx=4, n=16, length=1.0, mach=0.5, strength=5.0, radius=0.1,
                      dT=1e-3, sub_ratio=200.0, name="vortex") -> Case:
    """Inviscid isentropic vortex in a periodic box (ncx^3 cubes of n^3 cells).

    Free stream rho0=1.1842 kg/m^3, P0=101300 Pa (the reference's defaults,
    prm.h:27,37), U0 = mach * c0 along x.  Vortex of strength beta (in units
    of U0) and core radius `radius` centred in the box:
    u_theta = A r~ exp((1-r~^2)/2), A = beta U0 / (2 pi), r~ = r/radius;
    isentropic radial equilibrium gives T = T0 - A^2 exp(1-r~^2) / (2 cp).
    The field is formed with IEEE arithmetic only (exp_portable; the density
    power 1/(K-1) = 2.5 as t*t*sqrt(t)), so every machine builds the same
    bits and results can be compared with records made elsewhere.
    """
    ph = Phys(mu_L=0.0, rho0=1.1842, P0=101300.0, mpi_ncube=ncx ** 3)
    c0 = np.sqrt(GAMMA * ph.P0 / ph.rho0)
    ph.U0 = ph.Uin = mach * c0
    geom = periodic_box(ncx, ncx, ncx, n, length)
    X, Y, Z = _grid(geom, n)
    xc = yc = 0.5 * length
    dxr = (X - xc) / radius
    dyr = (Y - yc) / radius
    r2 = dxr * dxr + dyr * dyr
    A = strength * ph.U0 / (2 * np.pi)
    g = exp_portable(0.5 * (1 - r2))
    u = ph.U0 - A * dyr * g
    v = A * dxr * g
    w = np.zeros_like(u)
    cp = CV * GAMMA
    T0 = ph.P0 / (ph.rho0 * R_GAS)
    T = T0 - A * A * exp_portable(1 - r2) / (2 * cp)
    t = T / T0
    rho = ph.rho0 * (t * t * np.sqrt(t))  # (T/T0)^(1/(K-1)), K = 1.4
    p = rho * R_GAS * T
    U = conservative(rho, u, v, w, p)
    ncube, cube_size, csl, origin, adj = geom
    fws = np.full((ncube,) + (n + 4,) * 3, IFLUID, np.int32)
    return Case(n=n, ncube=ncube, phys=ph, cube_size=cube_size, csl=csl, origin=origin,
                adj=adj, fws=fws, U=np.ascontiguousarray(U), dT=dT, dTau=dT / sub_ratio,
                name=name)


def taylor_green(ncx=8, n=24, mach=0.1, reynolds=1600.0, dT=1e-4, sub_ratio=200.0,
                 name="tgv") -> Case:
    """Viscous Taylor-Green vortex in a periodic 2*pi box.

    u = U0 sin x cos y cos z, v = -U0 cos x sin y cos z, w = 0,
    p = P0 + rho0 U0^2/16 (cos 2x + cos 2y)(cos 2z + 2), rho = p/(R T0)
    (isothermal start).  U0 = mach * c0 and the Sutherland reference
    viscosity mu_L = rho0 U0 L / Re with L = 1 m.  dT and dTau default to the
    reference's run parameters (main.cpp:57-58).
    """
    ph = Phys(rho0=1.1842, P0=101300.0, mpi_ncube=ncx ** 3)
    c0 = np.sqrt(GAMMA * ph.P0 / ph.rho0)
    ph.U0 = ph.Uin = mach * c0
    ph.mu_L = ph.rho0 * ph.U0 * 1.0 / reynolds
    geom = periodic_box(ncx, ncx, ncx, n, 2 * np.pi)
    X, Y, Z = _grid(geom, n)
    U0 = ph.U0
    u = U0 * np.sin(X) * np.cos(Y) * np.cos(Z)
    v = -U0 * np.cos(X) * np.sin(Y) * np.cos(Z)
    w = np.zeros_like(u)
    p = ph.P0 + ph.rho0 * U0 * U0 / 16.0 * (np.cos(2 * X) + np.cos(2 * Y)) * (np.cos(2 * Z) + 2)
    T0 = ph.T0
    rho = p / (R_GAS * T0)
    U = conservative(rho, u, v, w, p)
    ncube, cube_size, csl, origin, adj = geom
    fws = np.full((ncube,) + (n + 4,) * 3, IFLUID, np.int32)
    return Case(n=n, ncube=ncube, phys=ph, cube_size=cube_size, csl=csl, origin=origin,
                adj=adj, fws=fws, U=np.ascontiguousarray(U), dT=dT, dTau=dT / sub_ratio,
                name=name)


def random_case(seed=1, ncx=2, ncy=2, ncz=2, n=4, periodic=False, viscous=True,
                solid_frac=0.08, ghost_frac=0.05, noise=0.05, with_ibm=True,
                name="random") -> Case:
    """Small stress case for parity: perturbed uniform flow, random
    fluid/ghost/solid flags (exercising every reconstruction fallback), open or
    periodic box (BCs visible when open) and random IBM ghost tables.

    Values stay physical (rho > 0, p > 0) so every branch is well defined.
    """
    ph = Phys(mu_L=0.0000185 if viscous else 0.0, rho0=1.1842, U0=38.889, Uin=38.889,
              P0=101300.0, mpi_ncube=ncx * ncy * ncz)
    geom = (periodic_box if periodic else open_box)(ncx, ncy, ncz, n, 1.0)
    ncube, cube_size, csl, origin, adj = geom
    S = n + 4
    cnt = ncube * S ** 3
    r = [splitmix_uniform(seed * 16 + t, cnt).reshape(ncube, S, S, S) for t in range(6)]
    rho = ph.rho0 * (1 + noise * (r[0] - 0.5))
    u = ph.U0 * (1 + 2 * noise * (r[1] - 0.5))
    v = ph.U0 * 2 * noise * (r[2] - 0.5)
    w = ph.U0 * 2 * noise * (r[3] - 0.5)
    p = ph.P0 * (1 + noise * 0.1 * (r[4] - 0.5))
    U = conservative(rho, u, v, w, p)
    fws = np.full((ncube, S, S, S), IFLUID, np.int32)
    fws[r[5] < solid_frac] = ISOLID
    fws[(r[5] >= solid_frac) & (r[5] < solid_frac + ghost_frac)] = IGHOST
    case = Case(n=n, ncube=ncube, phys=ph, cube_size=cube_size, csl=csl, origin=origin,
                adj=adj, fws=fws, U=np.ascontiguousarray(U), dT=1e-4, dTau=1e-4 / 200.0,
                name=name)
    if with_ibm:
        case.ibm_minus = random_ibm(seed * 16 + 7, case, count=6 * (ncube - 1))
        case.ibm_plus = random_ibm(seed * 16 + 9, case, count=4 * (ncube - 1))
    return case


def random_ibm(seed: int, case: Case, count: int):
    """Random IBM ghost tables (1-based packed).  Ghost cells are the case's
    IGHOST-flagged interior cells; image-point stencils (i..i+1, j..j+1,
    k..k+1) lie inside the padded cube.  About a quarter of entries put the
    ghost inside its own stencil, and some weights exceed 0.9999, so every
    special branch of BCM_Ghostcell_minus.cpp:192-449 runs.  Weights are
    rounded to 6 decimals like the reference's IBM files (%f)."""
    n, S = case.n, case.S
    ghosts = np.argwhere(case.fws[1:, 2:n + 2, 2:n + 2, 2:n + 2] == IGHOST)
    r = splitmix_uniform(seed, count * 16).reshape(count, 16)
    GC = np.zeros(4 * count + 1, np.int32)
    IP = np.zeros(4 * count + 1, np.int32)
    W = np.zeros(8 * count + 1)
    for e in range(count):
        if len(ghosts):
            g = ghosts[int(r[e, 0] * len(ghosts)) % len(ghosts)]
            gc, gi, gj, gk = int(g[0]) + 1, int(g[1]) + 2, int(g[2]) + 2, int(g[3]) + 2
        else:
            gc = 1 + int(r[e, 0] * (case.ncube - 1))
            gi, gj, gk = (2 + int(r[e, t] * n) for t in (1, 2, 3))
        if r[e, 4] < 0.25:
            # ghost inside its own stencil at offset (oi, oj, ok)
            oi, oj, ok = (int(r[e, t] * 2) for t in (5, 6, 7))
            ic, ii, jj, kk = gc, gi - oi, gj - oj, gk - ok
        else:
            ic = 1 + int(r[e, 5] * (case.ncube - 1))
            ii, jj, kk = (1 + int(r[e, t] * (S - 3)) for t in (6, 7, 8))
        w = r[e, 8:16] + 1e-3
        if r[e, 9] < 0.1:
            w[int(r[e, 10] * 8)] += 1e4  # one dominant weight (> 0.9999 after normalising)
        w = np.round(w / w.sum(), 6)
        GC[4 * e + 1:4 * e + 5] = (gc, gi, gj, gk)
        IP[4 * e + 1:4 * e + 5] = (ic, ii, jj, kk)
        W[8 * e + 1:8 * e + 9] = w
    return W, GC, IP


def two_level_box(ncx: int, ncy: int, ncz: int, n: int, length: float, refine, periodic=True):
    """Coarse cubes tiling [0, ncx*size) x ... in which every coarse cube with
    refine(a, b, c) true is replaced by 2x2x2 fine cubes (half size).

    Adjacency follows the reference's grid-file convention (BCM_Grid.cpp):
    adj[c][slot][dir], dir 1..6 = -x,+x,-y,+y,-z,+z.  A neighbour of equal or
    larger size sits in slot 1; the four smaller neighbours across a face sit
    in slots 1..4 ordered (lo,lo), (hi on the first tangential axis), (hi on
    the second), (hi,hi), tangential axes in x<y<z order (BCM_Interface.cpp
    :1825-1894).  csl = round(log2(size / smallest size)) (BCM_Grid.cpp:166).
    Returns (ncube, cube_size, csl, origin, adj).
    """
    size = length / ncx
    dims = (ncx, ncy, ncz)
    coarse_ref = {(a, b, c): bool(refine(a, b, c))
                  for a in range(ncx) for b in range(ncy) for c in range(ncz)}
    cubes = []  # (level, (i, j, k) in units of own size)
    for c in range(ncz):
        for b in range(ncy):
            for a in range(ncx):
                if coarse_ref[(a, b, c)]:
                    for dk in range(2):
                        for dj in range(2):
                            for di in range(2):
                                cubes.append((0, (2 * a + di, 2 * b + dj, 2 * c + dk)))
                else:
                    cubes.append((1, (a, b, c)))
    index = {cb: i + 1 for i, cb in enumerate(cubes)}
    ncube = len(cubes) + 1
    cube_size = np.zeros(ncube)
    csl = np.zeros(ncube, np.int32)
    origin = np.zeros((ncube, 3))
    adj = np.zeros((ncube, 5, 7), np.int32)

    def wrap(pos, lev):
        out = []
        for ax in range(3):
            m = dims[ax] * (2 if lev == 0 else 1)
            p = pos[ax]
            if periodic:
                p %= m
            elif p < 0 or p >= m:
                return None
            out.append(p)
        return tuple(out)

    for (lev, pos), ci in index.items():
        s = size if lev == 1 else size / 2
        cube_size[ci] = s
        csl[ci] = lev
        origin[ci] = [pos[0] * s, pos[1] * s, pos[2] * s]
        for ax in range(3):
            t0, t1 = [t for t in range(3) if t != ax]
            for sgn, d in ((-1, 1 + 2 * ax), (1, 2 + 2 * ax)):
                q = list(pos)
                q[ax] += sgn
                if lev == 0:
                    nb = wrap(q, 0)
                    if nb is None:
                        continue
                    if (0, nb) in index:
                        adj[ci, 1, d] = index[(0, nb)]
                    else:
                        cp = tuple(v // 2 for v in nb)
                        adj[ci, 1, d] = index[(1, cp)]
                else:
                    nb = wrap(q, 1)
                    if nb is None:
                        continue
                    if (1, nb) in index:
                        adj[ci, 1, d] = index[(1, nb)]
                    else:
                        # four fine cubes on the shared face
                        for slot, (h0, h1) in enumerate(((0, 0), (1, 0), (0, 1), (1, 1)), start=1):
                            f = [2 * v for v in nb]
                            f[ax] += 1 if sgn < 0 else 0  # fine layer touching this cube
                            f[t0] += h0
                            f[t1] += h1
                            adj[ci, slot, d] = index[(0, tuple(f))]
    return ncube, cube_size, csl, origin, adj


def random_two_level_case(seed=1, ncx=2, ncy=2, ncz=2, n=4, periodic=True, viscous=True,
                          noise=0.05, solid_frac=0.0, ghost_frac=0.0, name="two_level"):
    """Random perturbed flow on a two-level grid: coarse cube (0,0,0) of the
    ncx x ncy x ncz coarse tiling is refined into 8 fine cubes, so every face
    kind of the level-jump interface occurs (BCM_Interface.cpp:1790-4358)."""
    ph = Phys(mu_L=0.0000185 if viscous else 0.0, rho0=1.1842, U0=38.889, Uin=38.889,
              P0=101300.0, mpi_ncube=0)
    geom = two_level_box(ncx, ncy, ncz, n, 1.0, lambda a, b, c: (a, b, c) == (0, 0, 0),
                         periodic=periodic)
    ncube, cube_size, csl, origin, adj = geom
    ph.mpi_ncube = ncube - 1
    S = n + 4
    cnt = ncube * S ** 3
    r = [splitmix_uniform(seed * 16 + t, cnt).reshape(ncube, S, S, S) for t in range(6)]
    rho = ph.rho0 * (1 + noise * (r[0] - 0.5))
    u = ph.U0 * (1 + 2 * noise * (r[1] - 0.5))
    v = ph.U0 * 2 * noise * (r[2] - 0.5)
    w = ph.U0 * 2 * noise * (r[3] - 0.5)
    p = ph.P0 * (1 + noise * 0.1 * (r[4] - 0.5))
    U = conservative(rho, u, v, w, p)
    fws = np.full((ncube, S, S, S), IFLUID, np.int32)
    fws[r[5] < solid_frac] = ISOLID
    fws[(r[5] >= solid_frac) & (r[5] < solid_frac + ghost_frac)] = IGHOST
    return Case(n=n, ncube=ncube, phys=ph, cube_size=cube_size, csl=csl, origin=origin,
                adj=adj, fws=fws, U=np.ascontiguousarray(U), dT=1e-4, dTau=1e-4 / 200.0,
                name=name)


def icosphere(levels: int = 5, radius: float = 0.5, center=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Triangles [20 * 4**levels, 3, 3] of a sphere: an icosahedron whose faces
    are split into four `levels` times, new vertices pushed onto the sphere;
    counter-clockwise seen from outside (outward normals).  levels=5 gives the
    20,480 triangles of the sphere benchmark."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    verts = [np.array(v, np.float64) for v in (
        (-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t),
        (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1))]
    verts = [v / np.linalg.norm(v) for v in verts]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
             (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
             (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    tris = np.array([[verts[a], verts[b], verts[c]] for a, b, c in faces])
    for _ in range(levels):
        a, b, c = tris[:, 0], tris[:, 1], tris[:, 2]
        ab, bc, ca = a + b, b + c, c + a
        ab /= np.linalg.norm(ab, axis=1)[:, None]
        bc /= np.linalg.norm(bc, axis=1)[:, None]
        ca /= np.linalg.norm(ca, axis=1)[:, None]
        tris = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
                               np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)])
    return tris * radius + np.asarray(center, np.float64)


def write_stl(path: str, tris: np.ndarray, name: str = "body") -> None:
    """ASCII STL (the format BCM_Immersed_boundary.cpp:197-270 reads), every
    coordinate written so that it reads back exactly."""
    lines = [f"solid {name}"]
    for t in tris:
        nrm = np.cross(t[1] - t[0], t[2] - t[0])
        nrm = nrm / max(np.linalg.norm(nrm), 1e-300)
        lines.append("  facet normal %r %r %r" % tuple(float(x) for x in nrm))
        lines.append("    outer loop")
        for v in t:
            lines.append("      vertex %r %r %r" % tuple(float(x) for x in v))
        lines.append("    endloop")
        lines.append("  endfacet")
    lines.append(f"endsolid {name}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_stl(path: str) -> np.ndarray:
    """Triangles [ntri, 3, 3] of an ASCII STL, in file order."""
    vals = []
    with open(path) as f:
        for line in f:
            tok = line.split()
            if tok and tok[0] == "vertex":
                vals.append([float(x) for x in tok[1:4]])
    return np.asarray(vals, np.float64).reshape(-1, 3, 3)


def _pack_tables(gc, ip, w):
    """0-based [m,4] / [m,8] tables -> the 1-based packed arrays of
    BCM_Reading_IBM (weight[8m+1], GCindex[4m+1], IPsur[4m+1])."""
    m = len(gc)
    GC = np.zeros(4 * m + 1, np.int32)
    IP = np.zeros(4 * m + 1, np.int32)
    W = np.zeros(8 * m + 1)
    GC[1:] = np.asarray(gc, np.int32).reshape(-1)
    IP[1:] = np.asarray(ip, np.int32).reshape(-1)
    W[1:] = np.asarray(w, np.float64).reshape(-1)
    return W, GC, IP


def quantize_weights(w: np.ndarray) -> np.ndarray:
    """Weights as the reference's text files carry them (printed with %f, six
    decimals, then read back)."""
    return np.array([float("%f" % x) for x in np.asarray(w, np.float64).reshape(-1)]).reshape(
        np.shape(w))


def sphere_ibm(n=16, coarse=2.0, box=((-10.0, 20.0), (-10.0, 10.0), (-10.0, 10.0)),
               refine_box=((-2.0, 4.0), (-2.0, 2.0), (-2.0, 2.0)), diameter=1.0, mach=0.3,
               reynolds=300.0, noise=1e-4, seed=7, dT=1e-4, sub_ratio=200.0, name="sphere",
               preprocess=None, stl_levels=5):
    """Flow past a sphere with immersed-boundary ghost cells on a two-level grid.

    Coarse cubes of edge `coarse` tile `box`; those inside `refine_box` are
    split into 2x2x2 fine cubes (2:1).  Flags in the reference's convention
    (BCM.h:6-8): cells whose centre lies inside the sphere are solid; fluid
    cells with a solid face neighbour are IBM ghost cells, whose value the
    ghost fill sets halfway between the wall and an image point in the fluid
    (BCM_Ghostcell_minus.cpp:172-189 halves the velocity).

    IBM tables: with `preprocess` (a callable (case, triangles) -> (minus,
    plus), each (GCindex[m,4], IPsur[m,4], weight[m,8]) 0-based, updating
    case.fws in place like BCM_Immersed_boundary.cpp, e.g. the GPU
    preprocessing) they come from the icosphere of 20 * 4**stl_levels
    triangles (meta["triangles"]); without it, an analytic stand-in in the
    same convention: boundary point = the ghost centre's radial projection
    onto the sphere, image point = 2 centre - boundary point, trilinear
    weights of its 8 surrounding cells in the ghost's cube.  Weights are
    quantised to six decimals like the reference's files.  Free stream at
    `mach`, Re on the diameter, seeded density noise; solid cells at rest
    (BCM_Initial_condition.cpp).  Domain faces carry the reference's X/Y/Z
    boundary conditions.
    """
    (x0, x1), (y0, y1), (z0, z1) = box
    ncx, ncy, ncz = (int(round((x1 - x0) / coarse)), int(round((y1 - y0) / coarse)),
                     int(round((z1 - z0) / coarse)))
    (rx0, rx1), (ry0, ry1), (rz0, rz1) = refine_box

    def refine(a, b, c):
        cx0, cy0, cz0 = x0 + a * coarse, y0 + b * coarse, z0 + c * coarse
        return (cx0 >= rx0 - 1e-9 and cx0 + coarse <= rx1 + 1e-9 and cy0 >= ry0 - 1e-9 and
                cy0 + coarse <= ry1 + 1e-9 and cz0 >= rz0 - 1e-9 and cz0 + coarse <= rz1 + 1e-9)

    ncube, cube_size, csl, origin, adj = two_level_box(ncx, ncy, ncz, n, ncx * coarse, refine,
                                                       periodic=False)
    origin = origin + np.array([x0, y0, z0])
    S = n + 4
    ph = Phys(rho0=1.1842, P0=101300.0, mpi_ncube=ncube - 1)
    c0 = np.sqrt(GAMMA * ph.P0 / ph.rho0)
    ph.U0 = ph.Uin = mach * c0
    ph.mu_L = ph.rho0 * ph.U0 * diameter / reynolds
    R = 0.5 * diameter
    geom = (ncube, cube_size, csl, origin, adj)
    X, Y, Z = _grid(geom, n)
    r = np.sqrt(X * X + Y * Y + Z * Z)
    solid = r < R
    fws = np.where(solid, ISOLID, IFLUID).astype(np.int32)
    # ghost = fluid cell with a solid face neighbour (inside the padded cube)
    ghost = np.zeros_like(solid)
    for ax in (1, 2, 3):
        for sh in (1, -1):
            nb = np.roll(solid, sh, axis=ax)
            edge = [slice(None)] * 4
            edge[ax] = 0 if sh == 1 else S - 1
            nb[tuple(edge)] = False
            ghost |= (~solid) & nb
    fws[ghost] = IGHOST
    fws[0] = IFLUID
    cnt = ncube * S ** 3
    rnd = splitmix_uniform(seed, cnt).reshape(ncube, S, S, S)
    rho = ph.rho0 * (1 + noise * (rnd - 0.5))
    u = np.full_like(rho, ph.U0)
    zero = np.zeros_like(rho)
    p = np.full_like(rho, ph.P0)
    U = conservative(rho, u, zero, zero, p)
    rest = conservative(np.full_like(rho, ph.rho0), zero, zero, zero, p)
    U = np.where(solid[..., None], rest, U)
    case = Case(n=n, ncube=ncube, phys=ph, cube_size=cube_size, csl=csl, origin=origin, adj=adj,
                fws=fws, U=np.ascontiguousarray(U), dT=dT, dTau=dT / sub_ratio, name=name)
    if preprocess is not None:
        tris = icosphere(stl_levels, R)
        minus, plus = preprocess(case, tris)
        case.meta["triangles"] = len(tris)
    else:
        minus, plus = _analytic_sphere_tables(case, X, Y, Z, R)
    case.ibm_minus = _pack_tables(minus[0], minus[1], quantize_weights(minus[2]))
    case.ibm_plus = _pack_tables(plus[0], plus[1], quantize_weights(plus[2]))
    case.meta.update(area_ratio=2.602 / (np.pi / 4 * diameter ** 2),
                     ghosts=int((case.fws[1:] == IGHOST).sum()))
    return case


def _analytic_sphere_tables(case, X, Y, Z, R):
    """Analytic stand-in for the preprocessing in the reference convention
    (all entries on the minus side, as outward-facing geometry gives)."""
    n, S = case.n, case.n + 4
    gc, ip, ws = [], [], []
    idx = np.argwhere(case.fws[1:, 2:n + 2, 2:n + 2, 2:n + 2] == IGHOST)
    for cc, ii, jj, kk in idx:
        c, i, j, k = int(cc) + 1, int(ii) + 2, int(jj) + 2, int(kk) + 2
        dx = case.cube_size[c] / n
        xg = np.array([X[c, i, j, k], Y[c, i, j, k], Z[c, i, j, k]])
        bi = xg * (R / max(np.linalg.norm(xg), 1e-12))
        xi = 2 * xg - bi
        f = (xi - case.origin[c]) / dx + 1.5  # centre of cell m is origin + (m - 1.5) dx
        base = np.floor(f).astype(int)
        if np.any(base < 0) or np.any(base > S - 2):
            continue
        t = f - base
        wx, wy, wz = t
        w = np.array([(1 - wx) * (1 - wy) * (1 - wz), wx * (1 - wy) * (1 - wz),
                      (1 - wx) * wy * (1 - wz), (1 - wx) * (1 - wy) * wz, wx * wy * (1 - wz),
                      wx * (1 - wy) * wz, (1 - wx) * wy * wz, wx * wy * wz])
        gc.append((c, i, j, k))
        ip.append((c, int(base[0]), int(base[1]), int(base[2])))
        ws.append(w)
    m = len(gc)
    minus = (np.array(gc, np.int32).reshape(m, 4), np.array(ip, np.int32).reshape(m, 4),
             np.array(ws).reshape(m, 8))
    empty = (np.zeros((0, 4), np.int32), np.zeros((0, 4), np.int32), np.zeros((0, 8)))
    return minus, empty


def sphere_cubes(target, n=16, mach=0.3, reynolds=300.0, seed=7, dT=None, sub_ratio=200.0,
                 name=None, preprocess=None, stl_levels=5):
    """Sphere flow (D = 1, IBM ghost cells, two levels) with about `target`
    cubes: coarse cubes of edge 1 tile an mx x my x mz box (x about 1.5
    times y and z); the 2x2x2 coarse cubes around the sphere are split into
    64 fine cubes of edge 0.5, so the count is mx*my*mz + 56 (64 at least).
    dT defaults to a convective CFL of 0.5 on the fine cells.  preprocess,
    stl_levels: as sphere_ibm."""
    m = max(target - 56, 8)
    my = max(2, int(round((m / 1.5) ** (1.0 / 3.0))))
    mx = max(2, int(round(m / (my * my))))
    ix0 = max(0, min(mx - 2, mx // 3 - 1))
    iy0 = (my - 2) // 2
    x0, y0 = -(ix0 + 1.0), -(iy0 + 1.0)
    if dT is None:
        c0 = np.sqrt(GAMMA * 101300.0 / 1.1842)
        dT = 0.5 * (0.5 / n) / (mach * c0)
    return sphere_ibm(n=n, coarse=1.0, box=((x0, x0 + mx), (y0, y0 + my), (y0, y0 + my)),
                      refine_box=((-1.0, 1.0), (-1.0, 1.0), (-1.0, 1.0)), mach=mach,
                      reynolds=reynolds, seed=seed, dT=dT, sub_ratio=sub_ratio,
                      name=name or f"sphere{mx}x{my}x{my}", preprocess=preprocess,
                      stl_levels=stl_levels)


def sphere_batch(ncase=16, seed=2024, n=16, lo=64, hi=2048, preprocess=None, stl_levels=5):
    """Independent sphere flows for one batched context: cube counts drawn
    from the seed in [lo, hi] (realised to the nearest mx*my*mz + 56), Mach
    uniform in [0.1, 0.6], Re uniform in [100, 1000], per-case dT (CFL 0.5 on
    the fine cells) and per-case density-noise seeds.  preprocess,
    stl_levels: as sphere_ibm."""
    r = splitmix_uniform(seed, 3 * ncase).reshape(ncase, 3)
    out = []
    for q in range(ncase):
        target = lo + int(r[q, 0] * (hi - lo + 1))
        mach = 0.1 + 0.5 * float(r[q, 1])
        re = 100.0 + 900.0 * float(r[q, 2])
        out.append(sphere_cubes(min(target, hi), n=n, mach=mach, reynolds=re, seed=seed + 1 + q,
                                name=f"sphere{q}", preprocess=preprocess,
                                stl_levels=stl_levels))
    return out


class CaseBatch:
    """Cases advanced together in one batched context: `U` is the flat state
    of the batch (case q's cubes 1.. follow case q-1's; slot 0 unused), the
    layout bcmg_batch_create gives the device arrays."""

    def __init__(self, case_list, name="batch"):
        self.cases = list(case_list)
        self.n = self.cases[0].n
        self.name = name
        self.ncube = 1 + sum(c.ncube - 1 for c in self.cases)
        self.meta = {}
        self._U = None

    @property
    def n_cells(self) -> int:
        return sum(c.n_cells for c in self.cases)

    @property
    def U(self) -> np.ndarray:
        if self._U is None:
            S = self.n + 4
            U = np.zeros((self.ncube, S, S, S, 5))
            g = 1
            for c in self.cases:
                U[g:g + c.ncube - 1] = c.U[1:]
                g += c.ncube - 1
            self._U = U
        return self._U


def shard_plan(case, rank_of_cube, rank):
    """(own cubes, proxy cubes) of `rank` in a cube-sharded run, global
    numbers, from the library's planner (bcmg_shard_plan): the proxies are
    the remote cubes whose faces the rank's face tasks read."""
    import ctypes as C
    from . import _lib
    L = _lib.lib()
    adj = np.ascontiguousarray(case.adj, np.int32)
    csl = np.ascontiguousarray(case.csl, np.int32)
    rk = np.ascontiguousarray(rank_of_cube, np.int32)
    cap = case.ncube
    loc, prox = np.zeros(cap, np.int32), np.zeros(cap, np.int32)
    nl, npx = C.c_int(), C.c_int()
    r = L.bcmg_shard_plan(case.ncube, adj.ctypes.data, csl.ctypes.data, rk.ctypes.data,
                          int(rank), cap, C.byref(nl), loc.ctypes.data, C.byref(npx),
                          prox.ctypes.data)
    if r != 0:
        raise ValueError(f"bcmg_shard_plan failed ({r})")
    return loc[:nl.value].copy(), prox[:npx.value].copy()


def shard_bands(case, rank_of_cube, src, dst):
    """Face bands rank dst reads from rank src: [m, 4] (global source cube,
    axis, side of the source's face, layers), in the library's fixed order."""
    import ctypes as C
    from . import _lib
    L = _lib.lib()
    adj = np.ascontiguousarray(case.adj, np.int32)
    csl = np.ascontiguousarray(case.csl, np.int32)
    rk = np.ascontiguousarray(rank_of_cube, np.int32)
    nb = C.c_int()
    r = L.bcmg_shard_bands(case.ncube, adj.ctypes.data, csl.ctypes.data, rk.ctypes.data,
                           int(src), int(dst), 0, C.byref(nb), None)
    if r not in (0, -2):
        raise ValueError(f"bcmg_shard_bands failed ({r})")
    out = np.zeros(4 * max(nb.value, 1), np.int32)
    r = L.bcmg_shard_bands(case.ncube, adj.ctypes.data, csl.ctypes.data, rk.ctypes.data,
                           int(src), int(dst), nb.value, C.byref(nb), out.ctypes.data)
    if r != 0:
        raise ValueError(f"bcmg_shard_bands failed ({r})")
    return out[:4 * nb.value].reshape(-1, 4)


def shard_case(case, rank_of_cube, rank):
    """The case of one rank of a cube-sharded run (the reference's rank_map,
    main.cpp:576-596): its own cubes in slots 1..nlocal (ascending global
    numbers), then one proxy slot per remote cube its face tasks read;
    adjacency, sizes, levels, flags and state taken from the global case,
    adjacency entries mapped to local slots (0 for cubes of neither list),
    boundary lists and IBM tables of the own cubes only.  Returns (case,
    own cubes, proxy cubes)."""
    own, prox = shard_plan(case, rank_of_cube, rank)
    slots = np.concatenate([[0], own, prox]).astype(np.int64)
    g2l = np.zeros(case.ncube, np.int32)
    g2l[own] = np.arange(1, len(own) + 1)
    g2l[prox] = np.arange(len(own) + 1, len(own) + len(prox) + 1)
    adj = g2l[case.adj[slots]]
    adj[0] = 0
    cube_size = case.cube_size[slots].copy()
    cube_size[0] = case.cube_size[0]
    mine = np.zeros(case.ncube, bool)
    mine[own] = True
    bc = tuple(g2l[x[mine[x]]] for x in case.bc_lists())

    def ibm(t):
        if t is None:
            return None
        W, G, I = t
        m = (len(G) - 1) // 4
        gc, ip, w = G[1:].reshape(m, 4).copy(), I[1:].reshape(m, 4).copy(), W[1:].reshape(m, 8)
        if m and (gc[:, 0] != ip[:, 0]).any():
            # a rank fills the ghosts of its own cubes from their own cells
            raise ValueError("sharded runs need every IBM image-point stencil inside its ghost "
                             "cell's cube (as BCM_Immersed_boundary's tables are)")
        keep = mine[gc[:, 0]] if m else np.zeros(0, bool)
        gc, ip, w = gc[keep], ip[keep], w[keep]
        gc[:, 0] = g2l[gc[:, 0]]
        ip[:, 0] = g2l[ip[:, 0]]
        return _pack_tables(gc, ip, w)

    sub = Case(n=case.n, ncube=len(slots), phys=case.phys, cube_size=cube_size,
               csl=case.csl[slots].astype(np.int32), origin=case.origin[slots].copy(),
               adj=np.ascontiguousarray(adj, np.int32),
               fws=np.ascontiguousarray(case.fws[slots]), U=np.ascontiguousarray(case.U[slots]),
               dT=case.dT, dTau=case.dTau, e=case.e, name=f"{case.name}.rank{rank}",
               ibm_minus=ibm(case.ibm_minus), ibm_plus=ibm(case.ibm_plus), bc=bc)
    return sub, own, prox
