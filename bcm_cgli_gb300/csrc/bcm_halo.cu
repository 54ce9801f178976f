// Ghost-layer kernels around the flux: cube-to-cube interface, the X/Y/Z
// boundary conditions and the immersed-boundary ghost cells.
//
// All three are pure data movement plus a little FP64 arithmetic; each is
// organised so one CTA owns the cells it writes and only reads cells nobody
// writes during the launch, which makes every launch race-free and gives the
// reference's results exactly.
#include <cuda_runtime.h>

#include <algorithm>

#include "bcm_common.cuh"
#include "bcm_kernels.h"

namespace bcmg {

constexpr int kHaloThreads = 256;

// ---------------------------------------------------------------------------
// Interface (BCM_Interface.cpp).  Same-level faces (:1745-1783 x, :2608-2642
// y, :3478-3512 z) copy the neighbour's two interior layers into this cube's
// two ghost layers over the n x n face; every read is an interior cell, every
// write a ghost cell of the task's destination cube, so all face tasks run in
// parallel.  A second launch then averages the edge ghosts in the
// reference's three ordered phases (:5640-5732): i-edges, then j-edges, then
// k-edges.
// ---------------------------------------------------------------------------
// Level-jump faces (BCM_Interface.cpp:1790-2599 x, :2651-3470 y,
// :3518-4358 z).  Sub-face slot s offsets the tangential axes (x<y<z order)
// by ((s==2||s==4) n/2, (s==3||s==4) n/2).
//  kind 1, coarse -> fine: the small cube's two ghost layers facing the big
//    cube take the big cube's adjacent interior cell (n+1 or 2 along the
//    axis, (p/2+1, q/2+1) + slot offset across it), both layers alike;
//  kind 2, fine -> coarse: the big cube's two ghost layers over the slot's
//    quadrant take 0.125 * the sum of the small cube's 2x2x2 interior cells,
//    summed in the reference's order (000,100,010,001,110,101,011,111 in i,j,k).
// With a mirror (split precision) every written value's mirror value is
// written too: injections copy the source's, averages are converted.
__device__ __forceinline__ void level_face(const InterfaceArgs &a, int c, const FaceTask &ft) {
  const int n = a.n, S = n + 4, h = n / 2;
  const int ax = ft.axis;
  const int t0 = ax == 0 ? 1 : 0, t1 = ax == 2 ? 1 : 2;
  const int o0 = (ft.slot == 2 || ft.slot == 4) ? h : 0;
  const int o1 = (ft.slot == 3 || ft.slot == 4) ? h : 0;
  double *U = a.U1_;
  float *M = mirror_current(a.mir);
  double r0 = 0, e0 = 0;
  if (M) mirror_base(a.mir, a.bt, c, r0, e0);
  if (ft.kind == 1) {
    const int gs = ft.side == 0 ? n + 1 : 2;
    for (int w = threadIdx.x; w < 2 * n * n * 5; w += blockDim.x) {
      const int v = w % 5, cell = w / 5;
      const int l = cell / (n * n), p = 2 + (cell / n) % n, q = 2 + cell % n;
      int d[3], sr[3];
      d[ax] = ft.side == 0 ? l : n + 2 + l;
      d[t0] = p;
      d[t1] = q;
      sr[ax] = gs;
      sr[t0] = p / 2 + 1 + o0;
      sr[t1] = q / 2 + 1 + o1;
      const size_t od = 5 * cell_index(S, c, d[0], d[1], d[2]) + v;
      const size_t os = 5 * cell_index(S, ft.src, sr[0], sr[1], sr[2]) + v;
      U[od] = U[os];
      if (M) M[od] = M[os];
    }
  } else {
    for (int w = threadIdx.x; w < 2 * h * h * 5; w += blockDim.x) {
      const int v = w % 5, cell = w / 5;
      const int l = cell / (h * h), p = 2 + (cell / h) % h, q = 2 + cell % h;
      int d[3], b[3];
      d[ax] = ft.side == 1 ? n + 2 + l : l;
      d[t0] = p + o0;
      d[t1] = q + o1;
      b[ax] = ft.side == 1 ? 2 * (l + 1) : n - 2 + 2 * l;
      b[t0] = (p - 1) * 2;
      b[t1] = (q - 1) * 2;
      const double *B = U + 5 * cell_index(S, ft.src, b[0], b[1], b[2]) + v;
      const size_t si = (size_t)S * S * 5, sj = (size_t)S * 5, sk = 5;
      double sum = B[0];
      sum = sum + B[si];
      sum = sum + B[sj];
      sum = sum + B[sk];
      sum = sum + B[si + sj];
      sum = sum + B[si + sk];
      sum = sum + B[sj + sk];
      sum = sum + B[si + sj + sk];
      const size_t od = 5 * cell_index(S, c, d[0], d[1], d[2]) + v;
      U[od] = 0.125 * sum;
      if (M) M[od] = mirror_value_hw(0.125 * sum, v, r0, e0);
    }
  }
}

// Face copies: one CTA per (destination cube, face task).  Work items are
// (layer, row) pairs; a row is the n cells along the innermost index that
// both source and destination store contiguously (k for x and y faces), so
// lanes move consecutive doubles.  For z faces a row is one (i, j) column of
// the two ghost layers.
__global__ void __launch_bounds__(kHaloThreads) k_iface_faces(InterfaceArgs a) {
  const int n = a.n, S = n + 4;
  const int t = blockIdx.x;
  const int c = a.task_cube[t];
  if (!case_active(a.bt, c)) return;
  const FaceTask ft = a.tasks[t];
  const int ax = ft.axis;
  const int dbase = ft.side == 0 ? 0 : n + 2;
  const int sbase = ft.side == 0 ? n : 2;
  double *U = a.U1_;
  if (ft.kind != 0) {
    level_face(a, c, ft);
    return;
  }
  // Copies move pairs of values (16-byte pairs of doubles, 8-byte pairs of
  // mirror floats): S is even, so every row below starts at an even cell
  // index (an even value index) and is 5n or 10 values long (n is a multiple
  // of 4).  The mirror (split precision) is copied like the state: an exact
  // copy of a value has the same rounding.
  double2 *U2 = reinterpret_cast<double2 *>(U);
  float2 *M2 = reinterpret_cast<float2 *>(mirror_current(a.mir));
  // Source (the neighbour's interior) and destination (this cube's ghost
  // layers) never overlap: each thread issues its loads for kBatch items
  // before storing them, so the copies are not a chain of round trips.
  constexpr int kBatch = 4;
  auto copy = [&](int total, auto index) {
    for (int w0 = threadIdx.x; w0 < total; w0 += kBatch * kHaloThreads) {
      double2 u[kBatch];
      float2 m[kBatch];
      size_t od[kBatch];
#pragma unroll
      for (int b = 0; b < kBatch; ++b) {
        const int w = w0 + b * kHaloThreads;
        if (w < total) {
          size_t os;
          index(w, od[b], os);
          u[b] = U2[os];
          if (M2) m[b] = M2[os];
        }
      }
#pragma unroll
      for (int b = 0; b < kBatch; ++b)
        if (w0 + b * kHaloThreads < total) {
          U2[od[b]] = u[b];
          if (M2) M2[od[b]] = m[b];
        }
    }
  };
  if (ax < 2) {
    // rows: (layer l, transverse index p); each row = 5n doubles along k
    const int rowlen = 5 * n / 2;
    copy(2 * n * rowlen, [&](int w, size_t &od, size_t &os) {
      const int row = w / rowlen, e = w - row * rowlen;
      const int l = row / n, p = 2 + (row - l * n);
      int di, dj, si, sj;
      if (ax == 0) { di = dbase + l; si = sbase + l; dj = sj = p; }
      else { dj = dbase + l; sj = sbase + l; di = si = p; }
      od = 5 * cell_index(S, c, di, dj, 2) / 2 + e;
      os = 5 * cell_index(S, ft.src, si, sj, 2) / 2 + e;
    });
  } else {
    // z faces: per (i, j) the two layers are 10 contiguous doubles
    copy(n * n * 5, [&](int w, size_t &od, size_t &os) {
      const int col = w / 5, e = w - col * 5;
      const int i = 2 + col / n, j = 2 + (col - (col / n) * n);
      od = 5 * cell_index(S, c, i, j, dbase) / 2 + e;
      os = 5 * cell_index(S, ft.src, i, j, sbase) / 2 + e;
    });
  }
}

// Edge fill after all face copies (BCM_Interface.cpp:5640-5732).  The
// reference fills the layer-1 edge ghosts in three ordered phases: i-edges
// (i = 2..nx), then j-edges and k-edges over the whole ghost range, so the
// last two end at the corners.  Every edge cell that is not a corner reads
// two face ghosts (cells with one ghost coordinate), which no phase writes;
// the j-edge phase's corner values are overwritten by the k-edge phase
// before anything reads them; and the k-edge phase's corner value is the
// average of the j-edge and i-edge cells next to the corner, themselves
// averages of face ghosts.  So one pass computes each edge cell from two
// face ghosts and each corner from the two edge values it averages (formed
// from four face ghosts in registers): the reference's operations, the same
// bits, one round trip to memory instead of three dependent ones.  A thread
// issues the loads of kEdgeBatch items before their stores.
constexpr int kEdgeThreads = 256, kEdgeBatch = 4;

__global__ void __launch_bounds__(kEdgeThreads) k_iface_edges(InterfaceArgs a) {
  const int n = a.n, S = n + 4, nx = n + 1, nyy = n + 2;
  const int c = a.edge_list ? a.edge_cubes[blockIdx.x] : blockIdx.x + 1;
  if (!case_active(a.bt, c)) return;
  double *U = a.U1_;
  float *M = mirror_current(a.mir);
  double r0 = 0, e0 = 0;
  if (M) mirror_base(a.mir, a.bt, c, r0, e0);
  auto at = [&](int i, int j, int k, int v) { return 5 * cell_index(S, c, i, j, k) + v; };
  auto ghost = [&](int x) { return x == 1 || x == nyy; };
  auto in = [&](int x) { return x == 1 ? 2 : nx; };
  // an edge cell (two ghost coordinates): the average of its two inward
  // neighbours across its ghost axes, both face ghosts
  auto edge = [&](int i, int j, int k, int v) -> double {
    double p, q;
    if (!ghost(i)) { p = U[at(i, in(j), k, v)]; q = U[at(i, j, in(k), v)]; }
    else if (!ghost(j)) { p = U[at(in(i), j, k, v)]; q = U[at(i, j, in(k), v)]; }
    else { p = U[at(in(i), j, k, v)]; q = U[at(i, in(j), k, v)]; }
    return 0.5 * (p + q);
  };
  const int nedge = 12 * n, items = 5 * (nedge + 8);
  // the value and destination of item w
  auto item = [&](int w, double &r, size_t &d, int &v) {
    v = w % 5;
    const int cell = w / 5;
    int ci, cj, ck;
    if (cell < nedge) {
      // edge family f (free coordinate i, j or k = 2..nx) and its two ghost
      // coordinates
      const int f = cell / (4 * n), rem = cell - f * 4 * n;
      const int pos = 2 + (rem >> 2), g1 = (rem & 1) ? nyy : 1, g2 = (rem & 2) ? nyy : 1;
      if (f == 0) { ci = pos; cj = g1; ck = g2; }
      else if (f == 1) { ci = g1; cj = pos; ck = g2; }
      else { ci = g1; cj = g2; ck = pos; }
      r = edge(ci, cj, ck, v);
    } else {
      // corner: the k-edge phase's average of the j-edge cell and the i-edge
      // cell next to it
      const int q = cell - nedge;
      ci = (q & 1) ? nyy : 1; cj = (q & 2) ? nyy : 1; ck = (q & 4) ? nyy : 1;
      const double xj = edge(ci, in(cj), ck, v), yi = edge(in(ci), cj, ck, v);
      r = 0.5 * (xj + yi);
    }
    d = at(ci, cj, ck, v);
  };
  for (int w0 = threadIdx.x; w0 < items; w0 += kEdgeBatch * kEdgeThreads) {
    double r0v = 0, r1v = 0, r2v = 0, r3v = 0;
    size_t d0 = 0, d1 = 0, d2 = 0, d3 = 0;
    int v0 = 0, v1 = 0, v2 = 0, v3 = 0;
    const int w1 = w0 + kEdgeThreads, w2 = w0 + 2 * kEdgeThreads, w3 = w0 + 3 * kEdgeThreads;
    item(w0, r0v, d0, v0);
    if (w1 < items) item(w1, r1v, d1, v1);
    if (w2 < items) item(w2, r2v, d2, v2);
    if (w3 < items) item(w3, r3v, d3, v3);
    U[d0] = r0v;
    if (M) M[d0] = mirror_value_hw(r0v, v0, r0, e0);
    if (w1 < items) { U[d1] = r1v; if (M) M[d1] = mirror_value_hw(r1v, v1, r0, e0); }
    if (w2 < items) { U[d2] = r2v; if (M) M[d2] = mirror_value_hw(r2v, v2, r0, e0); }
    if (w3 < items) { U[d3] = r3v; if (M) M[d3] = mirror_value_hw(r3v, v3, r0, e0); }
  }
}

// ---------------------------------------------------------------------------
// Halo exchange of cube-sharded runs: the face bands a remote rank's face
// tasks read, gathered from this rank's cubes into a buffer, or scattered
// from a buffer into the proxy slots that stand for the remote cubes.  One
// CTA per band; a band's cells go in (layer, first in-face index, second)
// order, the in-face axes in x<y<z order.  Pure copies, so the proxies hold
// the remote cells bit for bit.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kHaloThreads)
    k_halo(double *U, Mirror mir, const int *bands, const long long *offs, long long total_cells,
           int n, double *bufU, int unpack) {
  float *M = mirror_current(mir);  // split precision: the current mirror too
  const int b = blockIdx.x;
  const int c = bands[4 * b], ax = bands[4 * b + 1], side = bands[4 * b + 2],
            L = bands[4 * b + 3];
  const int S = n + 4;
  const int t0 = ax == 0 ? 1 : 0, t1 = ax == 2 ? 1 : 2;
  const int l0 = side == 1 ? n + 2 - L : 2;  // first layer along the axis
  const long long o0 = offs[b];
  float *bufM = M ? reinterpret_cast<float *>(bufU + 5 * total_cells) : nullptr;
  const int cells = L * n * n;
  for (int w = threadIdx.x; w < cells * 5; w += blockDim.x) {
    const int v = w % 5, cell = w / 5;
    const int l = cell / (n * n), p = (cell / n) % n, q = cell % n;
    int x[3];
    x[ax] = l0 + l;
    x[t0] = 2 + p;
    x[t1] = 2 + q;
    const size_t g = 5 * cell_index(S, c, x[0], x[1], x[2]) + v;
    const size_t h = 5 * (size_t)(o0 + cell) + v;
    if (unpack) {
      U[g] = bufU[h];
      if (M) M[g] = bufM[h];
    } else {
      bufU[h] = U[g];
      if (M) bufM[h] = M[g];
    }
  }
}

cudaError_t launch_halo(double *U, const Mirror &mir, const int *bands, const long long *offs,
                        int nband, long long total_cells, int n, void *buf, int unpack,
                        cudaStream_t s) {
  if (nband <= 0) return cudaSuccess;
  k_halo<<<nband, kHaloThreads, 0, s>>>(U, mir, bands, offs, total_cells, n,
                                        static_cast<double *>(buf), unpack);
  return cudaGetLastError();
}

cudaError_t launch_interface(const InterfaceArgs &a, int ncubes_total, cudaStream_t s) {
  if (ncubes_total <= 1) return cudaSuccess;
  if (a.ntasks > 0) {
    k_iface_faces<<<a.ntasks, kHaloThreads, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const int ne = a.edge_list ? a.nedge : ncubes_total - 1;
  if (ne > 0) k_iface_edges<<<ne, kEdgeThreads, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Boundary conditions (BCM_X/Y/Z_boundary_condition.cpp) in one pass.  The
// reference fills the x faces (j, k interior: inflow from cell 2, zero
// gradient from cell nx), then the y faces over every i (zero gradient from
// row 2 / nx, interior k), then the z faces over every i, j (slip with w
// negated from plane 2, zero gradient from plane nx), in that order
// (main.cpp:1161-1165), so a y face's x-ghost rows copy values the x phase
// wrote and a z face copies both.  Each value a phase reads is, through at
// most two earlier phases, a copy or the inflow formula of a cell no phase
// writes: read() follows that chain.  So every ghost position is formed
// directly, with the reference's operations, in one pass with no barrier:
// the same bits (checked on the CPU against the ordered phases for every
// mask and axis subset, and by the GPU parity tests).  `axes` limits the
// pass to the faces of one twin call (the others' ghosts are then read as
// they are).
// ---------------------------------------------------------------------------
constexpr int kBcThreads = 256, kBcChunks = 8, kBcBatch = 4;

__global__ void __launch_bounds__(kBcThreads) k_bc(BcArgs a) {
  const int n = a.n, S = n + 4, nx = n + 1, nxx = n + 2, nxxx = n + 3;
  const int c = a.cubes[blockIdx.x];
  if (!case_active(a.bt, c)) return;
  const int m = a.masks[blockIdx.x];
  const int mx = (a.axes & 1) ? (m & 3) : 0, my = (a.axes & 2) ? ((m >> 2) & 3) : 0,
            mz = (a.axes & 4) ? ((m >> 4) & 3) : 0;
  double *U = a.U1_;
  // Split precision: the mirror values of every write, into both mirror
  // buffers.  The flux kernel writes the next buffer's interior cells and
  // same-level ghost layers, and the interface call after it the level-jump
  // layers and edges; the boundary layers are written here only, so the
  // next buffer takes them now and equals the state's rounding in every
  // cell once it becomes current.
  float *M = mirror_current(a.mir);
  float *Mo = M ? (M == a.mir.buf[0] ? a.mir.buf[1] : a.mir.buf[0]) : nullptr;
  double r0 = 0, e0 = 0;
  if (M) mirror_base(a.mir, a.bt, c, r0, e0);
  const double Uin = a.bt.cube_case ? a.bt.cases[a.bt.cube_case[c]].Uin : a.Uin;
  auto Q = [&](int i, int j, int k) { return U + 5 * cell_index(S, c, i, j, k); };
  auto interior = [&](int x) { return x >= 2 && x <= nx; };
  // component v of the inflow state (:43-80): rho and p from the cell,
  // u = Uin, v = w = 0
  auto inflow = [&](const double *q, int v) -> double {
    const double rho = q[0];
    if (v == 0) return rho;
    const double Uu = Uin, Vv = 0., Ww = 0;
    if (v == 1) return rho * Uu;
    if (v == 2) return rho * Vv;
    if (v == 3) return rho * Ww;
    const double U0 = q[1] / rho, V0 = q[2] / rho, W0 = q[3] / rho;
    double VV = U0 * U0 + V0 * V0 + W0 * W0;
    const double P = (q[4] - 0.5 * rho * VV) * (BCMG_K - 1);
    VV = Uu * Uu + Vv * Vv + Ww * Ww;
    return P / (BCMG_K - 1) + 0.5 * rho * VV;
  };
  // component v of cell (i, j, k) as the reference's order leaves it after
  // the x phase (upto 1) or after the x and y phases (upto 2)
  auto read = [&](int i, int j, int k, int upto, int v) -> double {
    if (upto >= 2 && my && interior(k)) {
      if ((my & 1) && j <= 1) j = 2;
      else if ((my & 2) && j >= nxx) j = nx;
    }
    if (mx && interior(j) && interior(k)) {
      if ((mx & 1) && i <= 1) return inflow(Q(2, j, k), v);
      if ((mx & 2) && i >= nxx) i = nx;
    }
    return Q(i, j, k)[v];
  };
  // ghost positions: x faces n^2 each, y faces S n each, z faces S^2 each;
  // each position fills both ghost layers with one value.  Items are
  // (position, component), component fastest, so a warp's loads and stores
  // run over whole cells in a row.
  const int cx = n * n, cy = S * n, cz = S * S;
  const int nxl = (mx & 1) ? cx : 0, nxu = (mx & 2) ? cx : 0, nyl = (my & 1) ? cy : 0,
            nyu = (my & 2) ? cy : 0, nzl = (mz & 1) ? cz : 0, nzu = (mz & 2) ? cz : 0;
  const int items = 5 * (nxl + nxu + nyl + nyu + nzl + nzu);
  // item w: its value and the offsets of its two destinations
  auto item = [&](int w, double &x, size_t &d1, size_t &d0) {
    const int v = w % 5;
    int q = w / 5;
    if (q < nxl) {
      const int j = 2 + q / n, k = 2 + q % n;
      x = inflow(Q(2, j, k), v);
      d1 = 5 * cell_index(S, c, 1, j, k) + v; d0 = 5 * cell_index(S, c, 0, j, k) + v;
      return;
    }
    q -= nxl;
    if (q < nxu) {
      const int j = 2 + q / n, k = 2 + q % n;
      x = Q(nx, j, k)[v];
      d1 = 5 * cell_index(S, c, nxx, j, k) + v; d0 = 5 * cell_index(S, c, nxxx, j, k) + v;
      return;
    }
    q -= nxu;
    if (q < nyl) {
      const int i = q / n, k = 2 + q % n;
      x = read(i, 2, k, 1, v);
      d1 = 5 * cell_index(S, c, i, 1, k) + v; d0 = 5 * cell_index(S, c, i, 0, k) + v;
      return;
    }
    q -= nyl;
    if (q < nyu) {
      const int i = q / n, k = 2 + q % n;
      x = read(i, nx, k, 1, v);
      d1 = 5 * cell_index(S, c, i, nxx, k) + v; d0 = 5 * cell_index(S, c, i, nxxx, k) + v;
      return;
    }
    q -= nyu;
    if (q < nzl) {  // slip wall: rho*w negated (:42-65)
      const int i = q / S, j = q % S;
      x = read(i, j, 2, 2, v);
      if (v == 3) x = -x;
      d1 = 5 * cell_index(S, c, i, j, 1) + v; d0 = 5 * cell_index(S, c, i, j, 0) + v;
      return;
    }
    q -= nzl;
    const int i = q / S, j = q % S;
    x = read(i, j, nx, 2, v);
    d1 = 5 * cell_index(S, c, i, j, nxx) + v; d0 = 5 * cell_index(S, c, i, j, nxxx) + v;
  };
  // kBcBatch items per round, all loaded before any is stored
  const int stride = gridDim.y * kBcThreads;
  for (int w0 = blockIdx.y * kBcThreads + threadIdx.x; w0 < items; w0 += kBcBatch * stride) {
    double x[kBcBatch];
    size_t d1[kBcBatch], d0[kBcBatch];
#pragma unroll
    for (int b = 0; b < kBcBatch; ++b)
      if (w0 + b * stride < items) item(w0 + b * stride, x[b], d1[b], d0[b]);
#pragma unroll
    for (int b = 0; b < kBcBatch; ++b)
      if (w0 + b * stride < items) {
        U[d1[b]] = x[b];
        U[d0[b]] = x[b];
        if (M) {
          const float mv = mirror_value_hw(x[b], (int)(d1[b] % 5), r0, e0);
          M[d1[b]] = mv; M[d0[b]] = mv; Mo[d1[b]] = mv; Mo[d0[b]] = mv;
        }
      }
  }
}

cudaError_t launch_bc(const BcArgs &a, int ncubes, cudaStream_t s) {
  if (ncubes <= 0) return cudaSuccess;
  k_bc<<<dim3(ncubes, kBcChunks), kBcThreads, 0, s>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// IBM ghost cells (BCM_Ghostcell_minus.cpp:72-489; _plus is identical).  One
// dependency level per launch: within a level no entry reads a cell another
// entry of the level writes, and the host orders the levels so every read
// sees exactly the value the reference's serial loop sees.
//
// Eight lanes per entry, one stencil cell each: a cell's primitives take
// three FP64 divisions, which on this part's narrow FP64 pipe dominate an
// entry's latency, so the eight cells run side by side; their weighted terms
// go through shared memory to the group's first lane, which sums them in
// the reference's order (000,100,010,001,110,101,011,111) and writes the
// ghost cell.  The levels are short, so the launch is latency-bound and
// this parallelism is what shortens it.
// ---------------------------------------------------------------------------
constexpr int kGhostThreads = 128, kGhostPer = kGhostThreads / 8;  // entries per CTA

__global__ void __launch_bounds__(kGhostThreads) k_ghost(GhostArgs a, int count) {
  // per entry and stencil cell: rho, p, u, v, w and the weighted density and
  // pressure deltas
  __shared__ double sh[kGhostPer][8][7];
  const int g = threadIdx.x >> 3, m = threadIdx.x & 7;
  const int t = blockIdx.x * kGhostPer + g;
  const bool live = t < count;
  const int e = live ? a.entries[t] : 0;
  const int S = a.n + 4;
  const int b = (e - 1) * 4;
  int c = 0, i = 0, j = 0, k = 0;
  bool act = false;
  if (live) {
    c = a.IPsur[b + 1]; i = a.IPsur[b + 2]; j = a.IPsur[b + 3]; k = a.IPsur[b + 4];
    act = case_active(a.bt, c);
  }
  double rho0 = a.rho0, P0 = a.P0;
  if (act && a.bt.cube_case) {  // the case of the stencil's cube
    const CaseConst &cq = a.bt.cases[a.bt.cube_case[c]];
    rho0 = cq.rho0;
    P0 = cq.P0;
  }
  if (act) {
    // cell m of the stencil, order 000,100,010,001,110,101,011,111 (:81-145)
    const int oi = (m == 1 || m == 4 || m == 5 || m == 7);
    const int oj = (m == 2 || m == 4 || m == 6 || m == 7);
    const int ok = (m == 3 || m == 5 || m == 6 || m == 7);
    const double *q = a.U1_ + 5 * cell_index(S, c, i + oi, j + oj, k + ok);
    const double rh = q[0];
    const double Uu = q[1] / rh, Vv = q[2] / rh, Ww = q[3] / rh;
    const double VV = Uu * Uu + Vv * Vv + Ww * Ww;
    const double Pp = (q[4] - 0.5 * rh * VV) * (BCMG_K - 1);
    double *o = sh[g][m];
    o[0] = rh; o[1] = Pp; o[2] = Uu; o[3] = Vv; o[4] = Ww;
  }
  __syncwarp();
  if (!act) return;
  const double(*X)[7] = sh[g];
  const int gc = a.GCindex[b + 1], gi = a.GCindex[b + 2], gj = a.GCindex[b + 3],
            gk = a.GCindex[b + 4];
  // Ghost inside its own stencil (:192-449); like the reference, only the
  // local indices are compared, not the cube.
  const int s = (gi - i) + 2 * (gj - j) + 4 * (gk - k);
  const bool self = (gi - i == 0 || gi - i == 1) && (gj - j == 0 || gj - j == 1) &&
                    (gk - k == 0 || gk - k == 1);
  // bit pattern (di,dj,dk) -> stencil slot in the 000,100,010,001,...
  // order (patterns 3 and 4 swap)
  const int sl = s == 3 ? 4 : (s == 4 ? 3 : s);
  // Lanes 0..4 form the weighted sums of one quantity each (density, p, u,
  // v, w), every sum in the reference's term order, into sh[g][q][5] (all
  // eight terms) and sh[g][q][6] (the seven terms without the ghost's own
  // slot, for a ghost inside its stencil).  On this part's narrow FP64 pipe
  // the five chains side by side take a fifth of the issue slots of one lane
  // forming all five.
  if (m < 5) {
    const double *w = a.weight + (size_t)(e - 1) * 8 + 1;
    double wl[8];
#pragma unroll
    for (int l = 0; l < 8; ++l) wl[l] = w[l];
    const double base = m == 0 ? rho0 : (m == 1 ? P0 : 0.0);
    auto term = [&](int l) { return m < 2 ? wl[l] * (X[l][m] - base) : wl[l] * X[l][m]; };
    double acc = term(0);
#pragma unroll
    for (int l = 1; l < 8; ++l) acc = acc + term(l);
    if (m < 2) acc = acc + base;
    sh[g][m][5] = acc;
    if (self) {
      const double wsl = wl[sl];
      double r;
      if (m < 2) {
        if (wsl > 0.9999) {
          r = X[sl][m];
        } else {
          double ar = 0;
          bool first = true;
          for (int l = 0; l < 8; ++l) {
            if (l == sl) continue;
            const double t = term(l);
            if (first) { ar = t; first = false; }
            else { ar = ar + t; }
          }
          r = ar / (1 - wsl) + base;
        }
      } else {
        double su = 0;
        bool first = true;
        for (int l = 0; l < 8; ++l) {
          if (l == sl) continue;
          const double t = term(l);
          if (first) { su = t; first = false; }
          else { su = su + t; }
        }
        r = su / (2 - wsl);
      }
      sh[g][m][6] = r;
    }
  }
  __syncwarp();
  if (m != 0) return;
  double o[5];
  if (!self) {
    const double rho = X[0][5], P = X[1][5], U = X[2][5], V = X[3][5], W = X[4][5];
    const double VV = U * U + V * V + W * W;
    o[0] = rho;
    o[1] = 0.5 * rho * U;
    o[2] = 0.5 * rho * V;
    o[3] = 0.5 * rho * W;
    o[4] = P / (BCMG_K - 1) + 0.5 * rho * 0.25 * VV;
  } else {
    const double r2 = X[0][6], p2 = X[1][6], U2 = X[2][6], V2 = X[3][6], W2 = X[4][6];
    const double VV2 = U2 * U2 + V2 * V2 + W2 * W2;
    o[0] = r2;
    o[1] = r2 * U2;
    o[2] = r2 * V2;
    o[3] = r2 * W2;
    o[4] = p2 / (BCMG_K - 1) + 0.5 * r2 * VV2;
  }
  const size_t go = 5 * cell_index(S, gc, gi, gj, gk);
  double *gp = a.U1_ + go;
#pragma unroll
  for (int v = 0; v < 5; ++v) gp[v] = o[v];
  if (float *M = mirror_current(a.mir)) {
    double r0, e0;
    mirror_base(a.mir, a.bt, gc, r0, e0);
#pragma unroll
    for (int v = 0; v < 5; ++v) M[go + v] = mirror_value_hw(o[v], v, r0, e0);
  }
}

cudaError_t launch_ghost(const GhostArgs &a, int count, cudaStream_t s, int priority) {
  if (count <= 0) return cudaSuccess;
  const unsigned grid = (count + kGhostPer - 1) / kGhostPer;
  if (priority == 0) {
    k_ghost<<<grid, kGhostThreads, 0, s>>>(a, count);
    return cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kGhostThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = priority;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_ghost, a, count);
}

}  // namespace bcmg
