// Immersed-boundary preprocessing on the GPU (BCM_Immersed_boundary.cpp
// :127-1081), a setup step: for every IBM ghost cell of the finest cubes it
// finds the boundary point on the body's surface triangles, the image point
// in the fluid and the trilinear weights of the image point's 8 surrounding
// cells, which the ghost fill uses every stage (BCM_Ghostcell_minus.cpp).
//
// The reference loops ghost cells x triangles on one core.  Here:
//  * k_ibm_keep: one thread per triangle tests its three vertices against
//    every cube's box widened by 1.5 cells (k_ibm_cube_box, :330-430);
//  * k_ibm_tri_prep: the ray invariants of every kept triangle, once;
//  * k_ibm_ray_part / k_ibm_ray_combine: ghost cells x triangle ranges
//    (triangles staged through shared memory, read by every thread of the
//    CTA), then per cell the first closest hit of a ray along each
//    triangle's normal over all ranges (:686-720, :1409-1450);
//  * k_ibm_closest_part / k_ibm_closest_combine: the same split for the
//    cells without any hit, the last closest point (:1290-1405);
//  * the side test of a cell uses the dotp of the last hit cell at or before
//    it in the reference's (cube, i, j, k) order, because the reference never
//    resets it; that carry is a short sequential pass on the host;
//  * k_ibm_weights: one thread per ghost cell forms the boundary and image
//    points, the distance test, the image point's base cell, the inverse of
//    the 8x8 Vandermonde matrix (Gauss-Jordan with partial pivoting) and the
//    eight weights (:759-1040).
// Every step keeps the reference's operation order and the translation unit
// is built with --fmad=false, so the tables equal the reference's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/bcm_gb300.h"
#include "bcm_common.cuh"
#include "bcm_kernels.h"
#include "bcm_trace.h"

namespace bcmg {
namespace {

constexpr double kMinimum = 0.0000001;  // prm.h `minimum`
constexpr double kBig = 100000000;       // prm.h `MAX`
constexpr int kTriChunk = 128;           // triangles staged per CTA pass

// Box of every cube widened by 1.5 cells, box[c*6 + 0..5] = x lo, x hi,
// y lo, y hi, z lo, z hi (the reference's bounds expressions, :330-430).
__global__ void k_ibm_cube_box(int ncube, int n, const double *__restrict__ cube_size,
                               const double *__restrict__ X, const double *__restrict__ Y,
                               const double *__restrict__ Z, double *__restrict__ box) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncube) return;
  const double dx = cube_size[c] / n;
  double *b = box + 6 * (size_t)c;
  b[0] = X[c] - 1.5 * dx; b[1] = X[c] + cube_size[c] + 1.5 * dx;
  b[2] = Y[c] - 1.5 * dx; b[3] = Y[c] + cube_size[c] + 1.5 * dx;
  b[4] = Z[c] - 1.5 * dx; b[5] = Z[c] + cube_size[c] + 1.5 * dx;
}

// keep[t] = 1 when a vertex of triangle t lies in some cube's widened box
// (cubes 1..ncube-1, staged through shared memory).
constexpr int kBoxChunk = 512;
__global__ void __launch_bounds__(256) k_ibm_keep(int ntri, const double *__restrict__ tri,
                                                  int ncube, const double *__restrict__ box,
                                                  int *__restrict__ keep) {
  __shared__ double sb[kBoxChunk * 6];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double v[9];
  for (int e = 0; e < 9; ++e) v[e] = t < ntri ? tri[9 * (size_t)t + e] : 0.0;
  int k = 0;
  for (int c0 = 1; c0 < ncube; c0 += kBoxChunk) {
    const int cnt = min(kBoxChunk, ncube - c0);
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * 6; e += blockDim.x) sb[e] = box[6 * (size_t)c0 + e];
    __syncthreads();
    if (k || t >= ntri) continue;
    for (int c = 0; c < cnt && !k; ++c) {
      const double *b = sb + 6 * c;
      for (int q = 0; q < 3; ++q)
        if (v[3 * q] >= b[0] && v[3 * q] <= b[1] && v[3 * q + 1] >= b[2] &&
            v[3 * q + 1] <= b[3] && v[3 * q + 2] >= b[4] && v[3 * q + 2] <= b[5]) {
          k = 1;
          break;
        }
    }
  }
  if (t < ntri) keep[t] = k;
}

// Closest point of a triangle (:1290-1405), with the interior weight formed
// as the reference forms it.
__device__ __forceinline__ void closest(const double *v, double x, double y, double z,
                                        double *p) {
  const double *a = v, *b = v + 3, *c = v + 6;
  const double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  const double ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  const double bc[3] = {c[0] - b[0], c[1] - b[1], c[2] - b[2]};
  const double ap[3] = {x - a[0], y - a[1], z - a[2]};
  const double d1 = ab[0] * ap[0] + ab[1] * ap[1] + ab[2] * ap[2];
  const double d2 = ac[0] * ap[0] + ac[1] * ap[1] + ac[2] * ap[2];
  if (d1 <= 0. && d2 <= 0.) { p[0] = a[0]; p[1] = a[1]; p[2] = a[2]; return; }
  const double bp[3] = {x - b[0], y - b[1], z - b[2]};
  const double d3 = ab[0] * bp[0] + ab[1] * bp[1] + ab[2] * bp[2];
  const double d4 = ac[0] * bp[0] + ac[1] * bp[1] + ac[2] * bp[2];
  if (d3 >= 0. && d4 <= d3) { p[0] = b[0]; p[1] = b[1]; p[2] = b[2]; return; }
  const double vc = d1 * d4 - d3 * d2;
  if (vc <= 0. && d1 >= 0. && d3 <= 0.) {
    const double w = d1 / (d1 - d3);
    p[0] = a[0] + w * ab[0]; p[1] = a[1] + w * ab[1]; p[2] = a[2] + w * ab[2];
    return;
  }
  const double cp[3] = {x - c[0], y - c[1], z - c[2]};
  const double d5 = ab[0] * cp[0] + ab[1] * cp[1] + ab[2] * cp[2];
  const double d6 = ac[0] * cp[0] + ac[1] * cp[1] + ac[2] * cp[2];
  if (d6 >= 0. && d5 <= d6) { p[0] = c[0]; p[1] = c[1]; p[2] = c[2]; return; }
  const double vb = d5 * d2 - d1 * d6;
  if (vb <= 0. && d2 >= 0. && d6 <= 0.) {
    const double w = d2 / (d2 - d6);
    p[0] = a[0] + w * ac[0]; p[1] = a[1] + w * ac[1]; p[2] = a[2] + w * ac[2];
    return;
  }
  const double va = d3 * d6 - d5 * d4;
  if (va <= 0. && (d4 - d3) >= 0. && (d5 - d6) >= 0.) {
    const double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    p[0] = b[0] + w * bc[0]; p[1] = b[1] + w * bc[1]; p[2] = b[2] + w * bc[2];
    return;
  }
  const double denom = 1. / (va + vb + vc);
  const double vv = vb * denom;
  const double w = vc + denom;
  p[0] = a[0] + ab[0] * vv + ac[0] * w;
  p[1] = a[1] + ab[1] * vv + ac[1] * w;
  p[2] = a[2] + ab[2] * vv + ac[2] * w;
}

// Ray invariants of one kept triangle (computed once; the same values the
// reference recomputes for every ghost cell): v0, e1 = v1 - v0, e2 = v2 - v0,
// the normal nu = e1 x e2, dir = -nu / |nu|, p = dir x e2, det = e1 . p,
// 1 / det and dir . dir.
constexpr int kRec = 22;
__global__ void k_ibm_tri_prep(int ntri, const double *__restrict__ tri,
                               double *__restrict__ rec) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntri) return;
  const double *v = tri + 9 * (size_t)t;
  double *r = rec + kRec * (size_t)t;
  const double e1[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
  const double e2[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
  const double nu[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                        e1[0] * e2[1] - e1[1] * e2[0]};
  const double dis = sqrt(nu[0] * nu[0] + nu[1] * nu[1] + nu[2] * nu[2]);
  const double dir[3] = {-nu[0] / dis, -nu[1] / dis, -nu[2] / dis};
  const double pp[3] = {dir[1] * e2[2] - dir[2] * e2[1], dir[2] * e2[0] - dir[0] * e2[2],
                        dir[0] * e2[1] - dir[1] * e2[0]};
  const double det = e1[0] * pp[0] + e1[1] * pp[1] + e1[2] * pp[2];
  for (int q = 0; q < 3; ++q) {
    r[q] = v[q];
    r[3 + q] = e1[q];
    r[6 + q] = e2[q];
    r[9 + q] = dir[q];
    r[12 + q] = pp[q];
    r[15 + q] = nu[q];
  }
  r[18] = det;
  r[19] = 1.0 / det;
  r[20] = dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2];
  r[21] = 0.0;
}

// Ray test of ghost centre o against triangle record r (Moller-Trumbore,
// :1409-1450: det below 1e-7 rejected, both directions accepted); on a hit
// returns 1 with tt = t.
__device__ __forceinline__ int ray_hit(const double *o, const double *r, double *tt) {
  if (r[18] < kMinimum) return 0;
  const double tv[3] = {o[0] - r[0], o[1] - r[1], o[2] - r[2]};
  const double u = tv[0] * r[12] + tv[1] * r[13] + tv[2] * r[14];
  if (u < 0.0 || u > r[18]) return 0;
  const double q[3] = {tv[1] * r[5] - tv[2] * r[4], tv[2] * r[3] - tv[0] * r[5],
                       tv[0] * r[4] - tv[1] * r[3]};
  const double w = r[9] * q[0] + r[10] * q[1] + r[11] * q[2];
  if (w < 0.0 || u + w > r[18]) return 0;
  *tt = (r[6] * q[0] + r[7] * q[1] + r[8] * q[2]) * r[19];
  return 1;
}

// Search over the kept triangles, split over CTAs: blockIdx.x picks 128
// ghost cells, blockIdx.y one of gridDim.y contiguous triangle ranges.  Per
// (range, ghost): the number of ray hits and the first triangle with the
// smallest |t| (dir . dir), the reference's strict `<` over its serial loop.
// Cells are a list (cell < 0: skipped) so the closest-point pass below can
// reuse the layout.
constexpr int kGhostBlock = 128;
__global__ void __launch_bounds__(kGhostBlock)
    k_ibm_ray_part(int ng, const double *__restrict__ cen, int ntri, int per,
                   const double *__restrict__ rec, int *__restrict__ hits_p,
                   int *__restrict__ best_p, double *__restrict__ nd_p) {
  __shared__ double st[kTriChunk * kRec];
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const bool has = g < ng;
  double o[3] = {0, 0, 0};
  if (has) { o[0] = cen[3 * g]; o[1] = cen[3 * g + 1]; o[2] = cen[3 * g + 2]; }
  const int t0 = blockIdx.y * per, t1 = min(ntri, t0 + per);
  int hits = 0, best = -1;
  double dmin = kBig;
  for (int base = t0; base < t1; base += kTriChunk) {
    const int cnt = min(kTriChunk, t1 - base);
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * kRec; e += blockDim.x)
      st[e] = rec[kRec * (size_t)base + e];
    __syncthreads();
    if (!has) continue;
    for (int t = 0; t < cnt; ++t) {
      double tt;
      if (!ray_hit(o, st + kRec * t, &tt)) continue;
      const double nd = fabs(tt) * st[kRec * t + 20];
      ++hits;
      if (nd < dmin) { dmin = nd; best = base + t; }
    }
  }
  if (!has) return;
  const size_t at = (size_t)blockIdx.y * ng + g;
  hits_p[at] = hits;
  best_p[at] = best;
  nd_p[at] = dmin;
}

// Per ghost cell: total hits; of the closest hit (smallest |t| dir.dir, the
// lowest triangle on ties) |t|, direction and dotp = nu . (v0 - centre),
// recomputed from that triangle with the same arithmetic.  out[g*8 + 0..5] =
// hits, |t|, d0, d1, d2, dotp.
__global__ void k_ibm_ray_combine(int ng, int nsplit, const double *__restrict__ cen,
                                  const double *__restrict__ rec,
                                  const int *__restrict__ hits_p, const int *__restrict__ best_p,
                                  const double *__restrict__ nd_p, double *__restrict__ out) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  int hits = 0, best = -1;
  double dmin = kBig;
  for (int sp = 0; sp < nsplit; ++sp) {
    const size_t at = (size_t)sp * ng + g;
    hits += hits_p[at];
    if (best_p[at] >= 0 && nd_p[at] < dmin) { dmin = nd_p[at]; best = best_p[at]; }
  }
  double tmin = kBig, d0 = 0, d1 = 0, d2 = 0, dotp = 0;
  if (best >= 0) {
    const double o[3] = {cen[3 * g], cen[3 * g + 1], cen[3 * g + 2]};
    const double *r = rec + kRec * (size_t)best;
    double tt = 0;
    ray_hit(o, r, &tt);
    tmin = fabs(tt);
    d0 = r[9]; d1 = r[10]; d2 = r[11];
    dotp = r[15] * (r[0] - o[0]) + r[16] * (r[1] - o[1]) + r[17] * (r[2] - o[2]);
  }
  double *w = out + 8 * (size_t)g;
  w[0] = hits; w[1] = tmin; w[2] = d0; w[3] = d1; w[4] = d2; w[5] = dotp;
}

// Closest-point search for the ghost cells without any hit (list[m] ghost
// numbers), split like the ray search: per (range, cell) the LAST triangle
// with the smallest squared distance (the reference's `<=`).
constexpr int kRawChunk = kTriChunk * kRec / 9;
__global__ void __launch_bounds__(kGhostBlock)
    k_ibm_closest_part(int m, const int *__restrict__ list, const double *__restrict__ cen,
                       int ntri, int per, const double *__restrict__ tri,
                       int *__restrict__ best_p, double *__restrict__ nd_p) {
  __shared__ double sv[kRawChunk * 9];
  const int e0 = blockIdx.x * blockDim.x + threadIdx.x;
  const bool has = e0 < m;
  double o[3] = {0, 0, 0};
  if (has) {
    const int g = list[e0];
    o[0] = cen[3 * g]; o[1] = cen[3 * g + 1]; o[2] = cen[3 * g + 2];
  }
  const int t0 = blockIdx.y * per, t1 = min(ntri, t0 + per);
  int best = -1;
  double dmin = kBig;
  for (int base = t0; base < t1; base += kRawChunk) {
    const int cnt = min(kRawChunk, t1 - base);
    __syncthreads();
    for (int e = threadIdx.x; e < cnt * 9; e += blockDim.x) sv[e] = tri[9 * (size_t)base + e];
    __syncthreads();
    if (!has) continue;
    for (int t = 0; t < cnt; ++t) {
      double p[3];
      closest(sv + 9 * t, o[0], o[1], o[2], p);
      const double nd = (p[0] - o[0]) * (p[0] - o[0]) + (p[1] - o[1]) * (p[1] - o[1]) +
                        (p[2] - o[2]) * (p[2] - o[2]);
      if (nd <= dmin) { dmin = nd; best = base + t; }
    }
  }
  if (!has) return;
  const size_t at = (size_t)blockIdx.y * m + e0;
  best_p[at] = best;
  nd_p[at] = dmin;
}

// The closest point of those cells (the highest triangle on ties) into
// out[g*8 + 2..4]; 0 when no triangle is within the search distance.
__global__ void k_ibm_closest_combine(int m, int nsplit, const int *__restrict__ list,
                                      const double *__restrict__ cen,
                                      const double *__restrict__ tri,
                                      const int *__restrict__ best_p,
                                      const double *__restrict__ nd_p, double *__restrict__ out) {
  const int e0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (e0 >= m) return;
  int best = -1;
  double dmin = kBig;
  for (int sp = 0; sp < nsplit; ++sp) {
    const size_t at = (size_t)sp * m + e0;
    if (best_p[at] >= 0 && nd_p[at] <= dmin) { dmin = nd_p[at]; best = best_p[at]; }
  }
  const int g = list[e0];
  double p[3] = {0, 0, 0};
  if (best >= 0) closest(tri + 9 * (size_t)best, cen[3 * g], cen[3 * g + 1], cen[3 * g + 2], p);
  double *w = out + 8 * (size_t)g;
  w[2] = p[0]; w[3] = p[1]; w[4] = p[2];
}

// Triangle ranges per ghost block so that a search launch fills the GPU
// (about 8 CTAs per SM), each range at least 64 triangles.
int ibm_splits(int nblocks, int ntri) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int want = (8 * sms + nblocks - 1) / nblocks;
  const int most = (ntri + 63) / 64;
  return std::max(1, std::min(want, most));
}

// In-place inverse of the 8x8 row-major matrix m (:1504-1576).
__device__ void invert8(double *m) {
  double a[8][8], b[8][8];
  for (int j = 0; j < 8; ++j)
    for (int i = 0; i < 8; ++i) {
      a[j][i] = m[i + 8 * j];
      b[j][i] = i == j ? 1.0 : 0.0;
    }
  for (int k = 0; k < 8; ++k) {
    int mx = k;
    for (int j = k + 1; j < 8; ++j)
      if (fabs(a[j][k]) > fabs(a[mx][k])) mx = j;
    if (mx != k)
      for (int i = 0; i < 8; ++i) {
        double t = a[mx][i]; a[mx][i] = a[k][i]; a[k][i] = t;
        t = b[mx][i]; b[mx][i] = b[k][i]; b[k][i] = t;
      }
    const double t = a[k][k];
    for (int i = 0; i < 8; ++i) { a[k][i] /= t; b[k][i] /= t; }
    for (int j = 0; j < 8; ++j)
      if (j != k) {
        const double f = a[j][k] / a[k][k];
        for (int i = 0; i < 8; ++i) {
          a[j][i] = a[j][i] - a[k][i] * f;
          b[j][i] = b[j][i] - b[k][i] * f;
        }
      }
  }
  for (int j = 0; j < 8; ++j)
    for (int i = 0; i < 8; ++i) m[i + 8 * j] = b[j][i];
}

// Per ghost cell: status (0 dropped, 1 turned fluid, 2 minus entry, 3 plus
// entry), the image point's base cell and the eight weights.
__global__ void __launch_bounds__(128) k_ibm_weights(int ng, int n, const int *__restrict__ gidx,
                                                     const double *__restrict__ cen,
                                                     const double *__restrict__ srch,
                                                     const double *__restrict__ dotp_eff,
                                                     const double *__restrict__ cube_size,
                                                     int ncube, const double *__restrict__ ctr,
                                                     int *__restrict__ status,
                                                     int *__restrict__ base,
                                                     double *__restrict__ weight) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ng) return;
  const int c = gidx[4 * g];
  const double o[3] = {cen[3 * g], cen[3 * g + 1], cen[3 * g + 2]};
  const double *r = srch + 8 * (size_t)g;
  const int hits = (int)r[0];
  const double tmin = r[1], d0 = r[2], d1 = r[3], d2 = r[4];
  const double dotp = dotp_eff[g];
  double BI[3], IP[3];
  if (dotp == 0) {
    for (int q = 0; q < 3; ++q) BI[q] = IP[q] = o[q];
  } else if (dotp > 0) {
    if (hits > 0) {
      BI[0] = o[0] - tmin * d0; BI[1] = o[1] - tmin * d1; BI[2] = o[2] - tmin * d2;
      IP[0] = o[0] + tmin * d0; IP[1] = o[1] + tmin * d1; IP[2] = o[2] + tmin * d2;
    } else {
      BI[0] = d0; BI[1] = d1; BI[2] = d2;
      for (int q = 0; q < 3; ++q) IP[q] = 2 * o[q] - BI[q];
    }
  } else {
    if (hits > 0) {
      BI[0] = o[0] + tmin * d0; BI[1] = o[1] + tmin * d1; BI[2] = o[2] + tmin * d2;
      IP[0] = o[0] - tmin * d0; IP[1] = o[1] - tmin * d1; IP[2] = o[2] - tmin * d2;
    } else {
      BI[0] = d0; BI[1] = d1; BI[2] = d2;
      for (int q = 0; q < 3; ++q) IP[q] = 2 * o[q] - BI[q];
    }
  }
  const double dx = cube_size[c] / n;
  const double dis = sqrt((BI[0] - o[0]) * (BI[0] - o[0]) + (BI[1] - o[1]) * (BI[1] - o[1]) +
                          (BI[2] - o[2]) * (BI[2] - o[2]));
  if (dis > sqrt(2.0) * dx) {
    status[g] = 1;
    return;
  }
  // cell centres of the cube along x, y, z (Xcnt, Ycnt, Zcnt)
  const int S = n + 4, nxx = n + 2;
  const double *cx = ctr + (size_t)c * S, *cy = ctr + ((size_t)ncube + c) * S,
               *cz = ctr + (2 * (size_t)ncube + c) * S;
  int ii, jj, kk, found = 0;
  for (ii = 0; ii <= nxx; ++ii)
    if (IP[0] >= cx[ii] && IP[0] <= cx[ii] + dx) { ++found; break; }
  for (jj = 0; jj <= nxx; ++jj)
    if (IP[1] >= cy[jj] && IP[1] <= cy[jj] + dx) { ++found; break; }
  for (kk = 0; kk <= nxx; ++kk)
    if (IP[2] >= cz[kk] && IP[2] <= cz[kk] + dx) { ++found; break; }
  if (found < 3) {
    status[g] = 0;
    return;
  }
  const double s1 = IP[0] - cx[ii], s2 = IP[1] - cy[jj], s3 = IP[2] - cz[kk];
  const double hx = cx[ii + 1] - cx[ii];
  const double hy = cy[jj + 1] - cy[jj];
  const double hz = cz[kk + 1] - cz[kk];
  // corners 000, 100, 010, 001, 110, 101, 011, 111
  const int ox[8] = {0, 1, 0, 0, 1, 1, 0, 1}, oy[8] = {0, 0, 1, 0, 1, 0, 1, 1},
            oz[8] = {0, 0, 0, 1, 0, 1, 1, 1};
  double V[64];
  for (int q = 0; q < 8; ++q) {
    const double sx = ox[q] ? hx : 0, sy = oy[q] ? hy : 0, sz = oz[q] ? hz : 0;
    V[q * 8 + 7] = 1;
    V[q * 8 + 6] = sz;
    V[q * 8 + 5] = sy;
    V[q * 8 + 4] = sx;
    V[q * 8 + 3] = sy * sz;
    V[q * 8 + 2] = sx * sz;
    V[q * 8 + 1] = sx * sy;
    V[q * 8 + 0] = sx * sy * sz;
  }
  invert8(V);
  bool ok = true;
  double w[8];
  for (int q = 0; q < 8; ++q) {
    w[q] = V[q] * s1 * s2 * s3 + V[q + 8] * s1 * s2 + V[q + 16] * s1 * s3 + V[q + 24] * s2 * s3 +
           V[q + 32] * s1 + V[q + 40] * s2 + V[q + 48] * s3 + V[q + 56];
    if (!(w[q] >= (-kMinimum) && w[q] <= (1 + kMinimum))) ok = false;
  }
  if (!ok) {
    status[g] = 0;
    return;
  }
  status[g] = dotp >= 0 ? 2 : 3;
  base[3 * g] = ii;
  base[3 * g + 1] = jj;
  base[3 * g + 2] = kk;
  for (int q = 0; q < 8; ++q) weight[8 * (size_t)g + q] = w[q];
}

template <typename T>
struct DevBuf {
  T *p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
  cudaError_t alloc(size_t count) { return cudaMalloc((void **)&p, sizeof(T) * (count ? count : 1)); }
};

}  // namespace
}  // namespace bcmg

using namespace bcmg;

namespace {

int fail(const std::string &m, int code) {
  bcmg_internal_set_error(m.c_str());
  return code;
}

#define CKI(expr)                                                                   \
  do {                                                                              \
    cudaError_t e__ = (expr);                                                       \
    if (e__ != cudaSuccess)                                                         \
      return fail(std::string(#expr) + ": " + cudaGetErrorString(e__), BCMG_ERR_CUDA); \
  } while (0)

}  // namespace

namespace {

// The preprocessing over a cell-centre table ctr[3][ncube][n+4] (x, y, z
// centres of every cube, BCM_Grid.cpp:124-148).
int ibm_run(int n, int ncube, const double *cube_size, const int *csl, const double *Xcube,
            const double *Ycube, const double *Zcube, const double *ctr, int *FWS, int ntri,
            const double *tri, int cap, int *nminus, int *gc_minus, int *ip_minus,
            double *w_minus, int *nplus, int *gc_plus, int *ip_plus, double *w_plus) {
  const int S = n + 4, nx = n + 1;
  // Ghost cells of the finest cubes, in (cube, i, j, k) order, and centres.
  std::vector<int> gidx;
  std::vector<double> cen;
  for (int c = 1; c < ncube; ++c) {
    if (csl[c] != 0) continue;
    if (!(cube_size[c] > 0)) return fail("cube_size must be positive", BCMG_ERR_ARG);
    for (int i = 2; i <= nx; ++i)
      for (int j = 2; j <= nx; ++j)
        for (int k = 2; k <= nx; ++k)
          if (FWS[cell_index(S, c, i, j, k)] == 0) {
            gidx.insert(gidx.end(), {c, i, j, k});
            cen.insert(cen.end(), {ctr[(size_t)c * S + i], ctr[((size_t)ncube + c) * S + j],
                                   ctr[(2 * (size_t)ncube + c) * S + k]});
          }
  }
  const int ng = (int)(gidx.size() / 4);
  if (ng == 0 || ntri == 0) return BCMG_OK;  // nothing to do
  DevBuf<double> dtri, dsize, dX, dY, dZ, dctr, dcen, drec, dsrch, ddot, dw;
  DevBuf<int> dkeep, dg, dstat, dbase;
  CKI(dtri.alloc((size_t)ntri * 9));
  CKI(dsize.alloc(ncube));
  CKI(dX.alloc(ncube));
  CKI(dY.alloc(ncube));
  CKI(dZ.alloc(ncube));
  CKI(dkeep.alloc(ntri));
  CKI(cudaMemcpy(dtri.p, tri, sizeof(double) * 9 * (size_t)ntri, cudaMemcpyHostToDevice));
  CKI(cudaMemcpy(dsize.p, cube_size, sizeof(double) * ncube, cudaMemcpyHostToDevice));
  CKI(cudaMemcpy(dX.p, Xcube, sizeof(double) * ncube, cudaMemcpyHostToDevice));
  CKI(cudaMemcpy(dY.p, Ycube, sizeof(double) * ncube, cudaMemcpyHostToDevice));
  CKI(cudaMemcpy(dZ.p, Zcube, sizeof(double) * ncube, cudaMemcpyHostToDevice));
  {
    DevBuf<double> dbox;
    CKI(dbox.alloc((size_t)6 * ncube));
    k_ibm_cube_box<<<(ncube + 127) / 128, 128>>>(ncube, n, dsize.p, dX.p, dY.p, dZ.p, dbox.p);
    CKI(cudaGetLastError());
    k_ibm_keep<<<(ntri + 255) / 256, 256>>>(ntri, dtri.p, ncube, dbox.p, dkeep.p);
    CKI(cudaGetLastError());
  }
  std::vector<int> keep(ntri);
  CKI(cudaMemcpy(keep.data(), dkeep.p, sizeof(int) * ntri, cudaMemcpyDeviceToHost));
  std::vector<double> kept;
  for (int t = 0; t < ntri; ++t)
    if (keep[t]) kept.insert(kept.end(), tri + 9 * (size_t)t, tri + 9 * (size_t)t + 9);
  const int nk = (int)(kept.size() / 9);
  if (nk == 0) return BCMG_OK;  // no triangle near any cube
  CKI(cudaMemcpy(dtri.p, kept.data(), sizeof(double) * kept.size(), cudaMemcpyHostToDevice));
  CKI(drec.alloc((size_t)nk * kRec));
  k_ibm_tri_prep<<<(nk + 127) / 128, 128>>>(nk, dtri.p, drec.p);
  CKI(cudaGetLastError());
  CKI(dcen.alloc(cen.size()));
  CKI(dg.alloc(gidx.size()));
  CKI(dsrch.alloc((size_t)ng * 8));
  CKI(cudaMemcpy(dcen.p, cen.data(), sizeof(double) * cen.size(), cudaMemcpyHostToDevice));
  CKI(cudaMemcpy(dg.p, gidx.data(), sizeof(int) * gidx.size(), cudaMemcpyHostToDevice));
  {
    const int gb = (ng + kGhostBlock - 1) / kGhostBlock;
    const int ns = ibm_splits(gb, nk), per = (nk + ns - 1) / ns;
    DevBuf<int> hp, bp;
    DevBuf<double> np_;
    CKI(hp.alloc((size_t)ns * ng));
    CKI(bp.alloc((size_t)ns * ng));
    CKI(np_.alloc((size_t)ns * ng));
    k_ibm_ray_part<<<dim3(gb, ns), kGhostBlock>>>(ng, dcen.p, nk, per, drec.p, hp.p, bp.p,
                                                  np_.p);
    CKI(cudaGetLastError());
    k_ibm_ray_combine<<<(ng + 127) / 128, 128>>>(ng, ns, dcen.p, drec.p, hp.p, bp.p, np_.p,
                                                 dsrch.p);
    CKI(cudaGetLastError());
  }
  // The side test's dotp carries over cells without a hit (in order).
  std::vector<double> srch((size_t)ng * 8), deff(ng);
  CKI(cudaMemcpy(srch.data(), dsrch.p, sizeof(double) * srch.size(), cudaMemcpyDeviceToHost));
  double carry = 0.0;
  std::vector<int> nohit;
  for (int g = 0; g < ng; ++g) {
    if (srch[8 * (size_t)g] > 0)
      carry = srch[8 * (size_t)g + 5];
    else
      nohit.push_back(g);
    deff[g] = carry;
  }
  // Closest points of the cells without a hit.
  if (!nohit.empty()) {
    const int m = (int)nohit.size();
    const int gb = (m + kGhostBlock - 1) / kGhostBlock;
    const int ns = ibm_splits(gb, nk), per = (nk + ns - 1) / ns;
    DevBuf<int> dl, bp;
    DevBuf<double> np_;
    CKI(dl.alloc(m));
    CKI(bp.alloc((size_t)ns * m));
    CKI(np_.alloc((size_t)ns * m));
    CKI(cudaMemcpy(dl.p, nohit.data(), sizeof(int) * m, cudaMemcpyHostToDevice));
    k_ibm_closest_part<<<dim3(gb, ns), kGhostBlock>>>(m, dl.p, dcen.p, nk, per, dtri.p, bp.p,
                                                      np_.p);
    CKI(cudaGetLastError());
    k_ibm_closest_combine<<<(m + 127) / 128, 128>>>(m, ns, dl.p, dcen.p, dtri.p, bp.p, np_.p,
                                                    dsrch.p);
    CKI(cudaGetLastError());
  }
  CKI(dctr.alloc((size_t)3 * ncube * S));
  CKI(ddot.alloc(ng));
  CKI(dstat.alloc(ng));
  CKI(dbase.alloc((size_t)ng * 3));
  CKI(dw.alloc((size_t)ng * 8));
  CKI(cudaMemcpy(dctr.p, ctr, sizeof(double) * 3 * (size_t)ncube * S, cudaMemcpyHostToDevice));
  CKI(cudaMemcpy(ddot.p, deff.data(), sizeof(double) * ng, cudaMemcpyHostToDevice));
  k_ibm_weights<<<(ng + 127) / 128, 128>>>(ng, n, dg.p, dcen.p, dsrch.p, ddot.p, dsize.p, ncube,
                                           dctr.p, dstat.p, dbase.p, dw.p);
  CKI(cudaGetLastError());
  std::vector<int> stat(ng), base((size_t)ng * 3);
  std::vector<double> w((size_t)ng * 8);
  CKI(cudaMemcpy(stat.data(), dstat.p, sizeof(int) * ng, cudaMemcpyDeviceToHost));
  CKI(cudaMemcpy(base.data(), dbase.p, sizeof(int) * base.size(), cudaMemcpyDeviceToHost));
  CKI(cudaMemcpy(w.data(), dw.p, sizeof(double) * w.size(), cudaMemcpyDeviceToHost));
  int cm = 0, cp = 0;
  for (int g = 0; g < ng; ++g) {
    cm += stat[g] == 2;
    cp += stat[g] == 3;
  }
  if (cm > cap || cp > cap) return fail("IBM table capacity exceeded", BCMG_ERR_ARG);
  if ((cm && (!gc_minus || !ip_minus || !w_minus)) || (cp && (!gc_plus || !ip_plus || !w_plus)))
    return fail("output table pointer missing", BCMG_ERR_ARG);
  for (int g = 0; g < ng; ++g) {
    const int *G = &gidx[4 * (size_t)g];
    if (stat[g] == 1) {
      FWS[cell_index(S, G[0], G[1], G[2], G[3])] = 1;  // boundary point too far: fluid
      continue;
    }
    if (stat[g] < 2) continue;
    const bool minus = stat[g] == 2;
    const int m = minus ? (*nminus)++ : (*nplus)++;
    int *GC = minus ? gc_minus : gc_plus, *IP = minus ? ip_minus : ip_plus;
    double *W = minus ? w_minus : w_plus;
    for (int q = 0; q < 4; ++q) GC[4 * m + q] = G[q];
    IP[4 * m] = G[0];
    for (int q = 0; q < 3; ++q) IP[4 * m + 1 + q] = base[3 * (size_t)g + q];
    for (int q = 0; q < 8; ++q) W[8 * m + q] = w[8 * (size_t)g + q];
  }
  return BCMG_OK;
}

}  // namespace

extern "C" int bcmg_ibm_preprocess(int n, int ncube, const double *cube_size, const int *csl,
                                   const double *Xcube, const double *Ycube, const double *Zcube,
                                   int *FWS, int ntri, const double *tri, int cap, int *nminus,
                                   int *gc_minus, int *ip_minus, double *w_minus, int *nplus,
                                   int *gc_plus, int *ip_plus, double *w_plus) {
  bcmg::TraceRange trace("bcmg_ibm_preprocess");
  bcmg_internal_set_error(nullptr);
  if (!nminus || !nplus) return fail("bad arguments", BCMG_ERR_ARG);
  *nminus = 0;
  *nplus = 0;
  if (n < 1 || ncube < 1 || !cube_size || !csl || !Xcube || !Ycube || !Zcube || !FWS ||
      ntri < 0 || (ntri > 0 && !tri) || cap < 0)
    return fail("bad arguments", BCMG_ERR_ARG);
  const int S = n + 4;
  // Cell centres as BCM_Grid.cpp:124-148 forms them.
  std::vector<double> ctr((size_t)3 * ncube * S, 0.0);
  const double *corner[3] = {Xcube, Ycube, Zcube};
  for (int a = 0; a < 3; ++a)
    for (int c = 1; c < ncube; ++c) {
      const double dx = cube_size[c] / n;
      for (int i = 0; i < S; ++i) ctr[((size_t)a * ncube + c) * S + i] = corner[a][c] + (i - 1.5) * dx;
    }
  return ibm_run(n, ncube, cube_size, csl, Xcube, Ycube, Zcube, ctr.data(), FWS, ntri, tri, cap,
                 nminus, gc_minus, ip_minus, w_minus, nplus, gc_plus, ip_plus, w_plus);
}

// ---------------------------------------------------------------------------
// Drop-in twin of BCM_Immersed_boundary (main.h:113-147, called at
// main.cpp:811): reads BCM_STL_fine.stl from the working directory with the
// reference's parsing (:197-270), runs the GPU preprocessing with the
// reference configuration's NcubeX, updates FWS and writes
// IBM_minus<myid>.dat / IBM_plus<myid>.dat exactly as :989-1047 does.  Cell
// centres come from Xcnt/Ycnt/Zcnt ([ncube][NcubeX+4] each, as the
// reference reads them); null arrays: formed from the cube corners like
// BCM_Grid.cpp:124-148.  Errors: bcmg_last_error() (the reference has no
// error path; a missing STL file is an error here).
// ---------------------------------------------------------------------------
extern "C" void BCM_Immersed_boundary(int myid, int ncube, int n_wallcube, int *NBC, double Xmin,
                                      double Xmax, double Ymin, double Ymax, double Zmin,
                                      double Zmax, double *cube_size, int *csl, double *Xcube,
                                      double *Ycube, double *Zcube, double *Xcnt, double *Ycnt,
                                      double *Zcnt, int *FWS, int *wallcube) {
  bcmg::TraceRange trace("BCM_Immersed_boundary");
  (void)n_wallcube; (void)NBC; (void)Xmin; (void)Xmax; (void)Ymin; (void)Ymax; (void)Zmin;
  (void)Zmax; (void)wallcube;
  bcmg_internal_set_error(nullptr);
  bcmg_reference_config cfg;
  bcmg_get_reference_config(&cfg);
  FILE *f = std::fopen("BCM_STL_fine.stl", "r");
  if (!f) { fail("cannot open BCM_STL_fine.stl", BCMG_ERR_ARG); return; }
  // Facets: after each token "normal", the normal, "outer loop vertex",
  // three coordinates, "vertex", three, "vertex", three.
  std::vector<double> tri;
  char tok[1024];
  while (std::fscanf(f, "%1023s", tok) == 1) {
    if (std::strstr("normal", tok) == nullptr) continue;
    double nv[3], v[9];
    char s1[1024], s2[1024], s3[1024], s4[1024], s5[1024];
    if (std::fscanf(f, "%lf%lf%lf%1023s%1023s%1023s%lf%lf%lf%1023s%lf%lf%lf%1023s%lf%lf%lf",
                    &nv[0], &nv[1], &nv[2], s1, s2, s3, &v[0], &v[1], &v[2], s4, &v[3], &v[4],
                    &v[5], s5, &v[6], &v[7], &v[8]) != 17)
      break;
    tri.insert(tri.end(), v, v + 9);
  }
  std::fclose(f);
  const int ntri = (int)(tri.size() / 9);
  const int n = cfg.ncube_x, S = n + 4;
  if (n < 1 || ncube < 1 || !cube_size || !csl || !Xcube || !Ycube || !Zcube || !FWS) {
    fail("bad arguments", BCMG_ERR_ARG);
    return;
  }
  std::vector<double> ctr((size_t)3 * ncube * S, 0.0);
  const double *cnt[3] = {Xcnt, Ycnt, Zcnt}, *corner[3] = {Xcube, Ycube, Zcube};
  for (int a = 0; a < 3; ++a)
    for (int c = 1; c < ncube; ++c) {
      const double dx = cube_size[c] / n;
      for (int i = 0; i < S; ++i)
        ctr[((size_t)a * ncube + c) * S + i] =
            cnt[a] ? cnt[a][(size_t)c * S + i] : corner[a][c] + (i - 1.5) * dx;
    }
  int cap = 1;
  for (size_t e = 0; e < (size_t)ncube * S * S * S; ++e) cap += FWS[e] == 0;
  std::vector<int> gm(4 * (size_t)cap), im(4 * (size_t)cap), gp(4 * (size_t)cap),
      ipp(4 * (size_t)cap);
  std::vector<double> wm(8 * (size_t)cap), wp(8 * (size_t)cap);
  int nm = 0, np = 0;
  if (ibm_run(n, ncube, cube_size, csl, Xcube, Ycube, Zcube, ctr.data(), FWS, ntri, tri.data(),
              cap, &nm, gm.data(), im.data(), wm.data(), &np, gp.data(), ipp.data(),
              wp.data()) != BCMG_OK)
    return;
  for (int side = 0; side < 2; ++side) {
    char name[64];
    std::snprintf(name, sizeof name, side == 0 ? "IBM_plus%05d.dat" : "IBM_minus%05d.dat", myid);
    FILE *o = std::fopen(name, "w");
    if (!o) { fail(std::string("cannot write ") + name, BCMG_ERR_ARG); return; }
    const int m = side == 0 ? np : nm;
    const int *G = side == 0 ? gp.data() : gm.data(), *I = side == 0 ? ipp.data() : im.data();
    const double *W = side == 0 ? wp.data() : wm.data();
    for (int e = 0; e < m; ++e) {
      std::fprintf(o, "%d\t%d\t%d\t%d\n", G[4 * e], G[4 * e + 1], G[4 * e + 2], G[4 * e + 3]);
      std::fprintf(o, "%d\t%d\t%d\t%d\n", I[4 * e], I[4 * e + 1], I[4 * e + 2], I[4 * e + 3]);
      std::fprintf(o, "%f\t%f\t%f\t%f\t%f\t%f\t%f\t%f\n", W[8 * e], W[8 * e + 1], W[8 * e + 2],
                   W[8 * e + 3], W[8 * e + 4], W[8 * e + 5], W[8 * e + 6], W[8 * e + 7]);
    }
    std::fprintf(o, "Number of Boundary Cells\n");
    std::fprintf(o, "%d", m);
    std::fclose(o);
  }
}
