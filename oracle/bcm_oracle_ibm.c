/*
 * ORACLE (test infrastructure; never part of the product path).
 *
 * Immersed-boundary preprocessing of BCM_Immersed_boundary.cpp:127-1081
 * restated in plain C (serial, the reference's operation order; built with
 * -ffp-contract=off), the checker for the GPU preprocessing.  Pinned against
 * the reference's own compiled routine (tests/test_ibm_oracle.py).
 *
 * Input triangles are the STL facets in file order (three vertices each;
 * the facet normal of the file is not used, :232-260).  Steps:
 *  1. keep the triangles with any vertex inside some cube's box widened by
 *     1.5 cells (:330-430), in order;
 *  2. ghost cells: interior cells flagged IGHOST of the finest cubes
 *     (csl == 0), in (cube, i, j, k) order (:587-620);
 *  3. per ghost cell, every kept triangle in order: a ray from the cell
 *     centre along the triangle's normal (Moller-Trumbore, det below 1e-7
 *     rejected, both directions accepted); the first closest hit gives the
 *     boundary point; with no hit, the last closest point over all
 *     triangles (:686-720, :1086-1405);
 *  4. the side test uses dotp = n . (v0 - centre) of the closest hit; a
 *     cell without any hit keeps the previous cell's dotp (the reference
 *     never resets it; 0 before the first hit);
 *  5. boundary point BI and image point IP = 2 centre - BI (:759-855);
 *     |BI - centre| > sqrt(2) dx turns the cell fluid (:868-874); an image
 *     point outside the cube's cell range drops the cell (:886-920);
 *  6. trilinear weights by inverting the 8x8 Vandermonde matrix of the
 *     surrounding cells (Gauss-Jordan with partial pivoting, :934-975,
 *     :1504-1576); all eight in [-1e-7, 1 + 1e-7] -> an entry of the minus
 *     table (dotp >= 0) or the plus table (:989-1040).
 */
#include <math.h>
#include <stddef.h>

#include "bcm_oracle.h"

#define IGHOST 0
#define IFLUID 1
#define MINIMUM 0.0000001
#define BIG 100000000

static inline size_t at(int S, int c, int i, int j, int k) {
  return ((((size_t)c * S + i) * S + j) * S + k);
}

/* Moller-Trumbore as :1409-1450 (t, u, v set only on a hit). */
static int intersect(const double *orig, const double *dir, const double *v0, const double *v1,
                     const double *v2, double *t) {
  double e1[3] = {v1[0] - v0[0], v1[1] - v0[1], v1[2] - v0[2]};
  double e2[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
  double p[3] = {dir[1] * e2[2] - dir[2] * e2[1], dir[2] * e2[0] - dir[0] * e2[2],
                 dir[0] * e2[1] - dir[1] * e2[0]};
  double det = e1[0] * p[0] + e1[1] * p[1] + e1[2] * p[2];
  if (det < MINIMUM) return 0;
  double tv[3] = {orig[0] - v0[0], orig[1] - v0[1], orig[2] - v0[2]};
  double u = tv[0] * p[0] + tv[1] * p[1] + tv[2] * p[2];
  if (u < 0.0 || u > det) return 0;
  double q[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2],
                 tv[0] * e1[1] - tv[1] * e1[0]};
  double v = dir[0] * q[0] + dir[1] * q[1] + dir[2] * q[2];
  if (v < 0.0 || u + v > det) return 0;
  double tt = e2[0] * q[0] + e2[1] * q[1] + e2[2] * q[2];
  double inv = 1.0 / det;
  *t = tt * inv;
  return 1;
}

/* Closest point of a triangle (:1290-1405), including its interior-region
 * weight w = vc + denom as the reference forms it. */
static void closest(const double *a, const double *b, const double *c, double x, double y,
                    double z, double *p) {
  double ab[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
  double ac[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
  double bc[3] = {c[0] - b[0], c[1] - b[1], c[2] - b[2]};
  double ap[3] = {x - a[0], y - a[1], z - a[2]};
  double d1 = ab[0] * ap[0] + ab[1] * ap[1] + ab[2] * ap[2];
  double d2 = ac[0] * ap[0] + ac[1] * ap[1] + ac[2] * ap[2];
  if (d1 <= 0. && d2 <= 0.) { p[0] = a[0]; p[1] = a[1]; p[2] = a[2]; return; }
  double bp[3] = {x - b[0], y - b[1], z - b[2]};
  double d3 = ab[0] * bp[0] + ab[1] * bp[1] + ab[2] * bp[2];
  double d4 = ac[0] * bp[0] + ac[1] * bp[1] + ac[2] * bp[2];
  if (d3 >= 0. && d4 <= d3) { p[0] = b[0]; p[1] = b[1]; p[2] = b[2]; return; }
  double vc = d1 * d4 - d3 * d2;
  if (vc <= 0. && d1 >= 0. && d3 <= 0.) {
    double v = d1 / (d1 - d3);
    p[0] = a[0] + v * ab[0]; p[1] = a[1] + v * ab[1]; p[2] = a[2] + v * ab[2];
    return;
  }
  double cp[3] = {x - c[0], y - c[1], z - c[2]};
  double d5 = ab[0] * cp[0] + ab[1] * cp[1] + ab[2] * cp[2];
  double d6 = ac[0] * cp[0] + ac[1] * cp[1] + ac[2] * cp[2];
  if (d6 >= 0. && d5 <= d6) { p[0] = c[0]; p[1] = c[1]; p[2] = c[2]; return; }
  double vb = d5 * d2 - d1 * d6;
  if (vb <= 0. && d2 >= 0. && d6 <= 0.) {
    double w = d2 / (d2 - d6);
    p[0] = a[0] + w * ac[0]; p[1] = a[1] + w * ac[1]; p[2] = a[2] + w * ac[2];
    return;
  }
  double va = d3 * d6 - d5 * d4;
  if (va <= 0. && (d4 - d3) >= 0. && (d5 - d6) >= 0.) {
    double w = (d4 - d3) / ((d4 - d3) + (d5 - d6));
    p[0] = b[0] + w * bc[0]; p[1] = b[1] + w * bc[1]; p[2] = b[2] + w * bc[2];
    return;
  }
  double denom = 1. / (va + vb + vc);
  double v = vb * denom;
  double w = vc + denom;
  p[0] = a[0] + ab[0] * v + ac[0] * w;
  p[1] = a[1] + ab[1] * v + ac[1] * w;
  p[2] = a[2] + ab[2] * v + ac[2] * w;
}

/* In-place inverse of the 8x8 matrix m (row-major), :1504-1576. */
static void invert8(double *m) {
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
    double t = a[k][k];
    for (int i = 0; i < 8; ++i) { a[k][i] /= t; b[k][i] /= t; }
    for (int j = 0; j < 8; ++j)
      if (j != k) {
        double f = a[j][k] / a[k][k];
        for (int i = 0; i < 8; ++i) {
          a[j][i] = a[j][i] - a[k][i] * f;
          b[j][i] = b[j][i] - b[k][i] * f;
        }
      }
  }
  for (int j = 0; j < 8; ++j)
    for (int i = 0; i < 8; ++i) m[i + 8 * j] = b[j][i];
}

int bcmo_ibm(int n, int ncube, const double *cube_size, const int *csl, const double *Xcube,
             const double *Ycube, const double *Zcube, int *FWS, int ntri_in, const double *tri_in,
             int cap, int *nminus, int *gc_m, int *ip_m, double *w_m, int *nplus, int *gc_p,
             int *ip_p, double *w_p, double *tri_scratch) {
  const int S = n + 4, nx = n + 1, nxx = n + 2;
  /* 1. triangles with a vertex inside some widened cube box, in order */
  int ntri = 0;
  for (int t = 0; t < ntri_in; ++t) {
    const double *v = tri_in + 9 * t;
    int keep = 0;
    for (int q = 0; q < 3 && !keep; ++q)
      for (int c = 1; c < ncube; ++c) {
        double dx = cube_size[c] / n;
        double px = v[3 * q], py = v[3 * q + 1], pz = v[3 * q + 2];
        if (px >= Xcube[c] - 1.5 * dx && px <= Xcube[c] + cube_size[c] + 1.5 * dx &&
            py >= Ycube[c] - 1.5 * dx && py <= Ycube[c] + cube_size[c] + 1.5 * dx &&
            pz >= Zcube[c] - 1.5 * dx && pz <= Zcube[c] + cube_size[c] + 1.5 * dx) {
          keep = 1;
          break;
        }
      }
    if (keep) {
      for (int e = 0; e < 9; ++e) tri_scratch[9 * ntri + e] = v[e];
      ++ntri;
    }
  }
  *nminus = 0;
  *nplus = 0;
  double dotp = 0.0; /* carried from ghost cell to ghost cell */
  for (int c = 1; c < ncube; ++c) {
    if (csl[c] != 0) continue;
    const double dx = cube_size[c] / n;
    for (int gi = 2; gi <= nx; ++gi)
      for (int gj = 2; gj <= nx; ++gj)
        for (int gk = 2; gk <= nx; ++gk) {
          if (FWS[at(S, c, gi, gj, gk)] != IGHOST) continue;
          if (ntri == 0) continue;
          double o[3] = {Xcube[c] + (gi - 1.5) * dx, Ycube[c] + (gj - 1.5) * dx,
                         Zcube[c] + (gk - 1.5) * dx};
          int hits = 0;
          double tmin = BIG, dmin = BIG, d0 = 0, d1 = 0, d2 = 0;
          for (int t = 0; t < ntri; ++t) {
            const double *v = tri_scratch + 9 * t;
            double e12[3] = {v[3] - v[0], v[4] - v[1], v[5] - v[2]};
            double e13[3] = {v[6] - v[0], v[7] - v[1], v[8] - v[2]};
            double nu[3] = {e12[1] * e13[2] - e12[2] * e13[1], e12[2] * e13[0] - e12[0] * e13[2],
                            e12[0] * e13[1] - e12[1] * e13[0]};
            double dis = sqrt(nu[0] * nu[0] + nu[1] * nu[1] + nu[2] * nu[2]);
            double dir[3] = {-nu[0] / dis, -nu[1] / dis, -nu[2] / dis};
            double tt = 0;
            int hit = intersect(o, dir, v, v + 3, v + 6, &tt);
            double nd = fabs(tt) * (dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
            if (hit) {
              ++hits;
              if (nd < dmin) {
                dmin = nd;
                tmin = fabs(tt);
                d0 = dir[0]; d1 = dir[1]; d2 = dir[2];
                dotp = nu[0] * (v[0] - o[0]) + nu[1] * (v[1] - o[1]) + nu[2] * (v[2] - o[2]);
              }
            }
          }
          double bp[3] = {0, 0, 0};
          if (hits == 0) {
            dmin = BIG;
            for (int t = 0; t < ntri; ++t) {
              const double *v = tri_scratch + 9 * t;
              double p[3];
              closest(v, v + 3, v + 6, o[0], o[1], o[2], p);
              double nd = (p[0] - o[0]) * (p[0] - o[0]) + (p[1] - o[1]) * (p[1] - o[1]) +
                          (p[2] - o[2]) * (p[2] - o[2]);
              if (nd <= dmin) { bp[0] = p[0]; bp[1] = p[1]; bp[2] = p[2]; dmin = nd; }
            }
          }
          double BI[3], IP[3];
          if (dotp == 0) {
            for (int q = 0; q < 3; ++q) BI[q] = IP[q] = o[q];
          } else if (dotp > 0) {
            if (hits > 0) {
              BI[0] = o[0] - tmin * d0; BI[1] = o[1] - tmin * d1; BI[2] = o[2] - tmin * d2;
              IP[0] = o[0] + tmin * d0; IP[1] = o[1] + tmin * d1; IP[2] = o[2] + tmin * d2;
            } else {
              for (int q = 0; q < 3; ++q) { BI[q] = bp[q]; IP[q] = 2 * o[q] - BI[q]; }
            }
          } else {
            if (hits > 0) {
              BI[0] = o[0] + tmin * d0; BI[1] = o[1] + tmin * d1; BI[2] = o[2] + tmin * d2;
              IP[0] = o[0] - tmin * d0; IP[1] = o[1] - tmin * d1; IP[2] = o[2] - tmin * d2;
            } else {
              for (int q = 0; q < 3; ++q) { BI[q] = bp[q]; IP[q] = 2 * o[q] - BI[q]; }
            }
          }
          double dis = sqrt((BI[0] - o[0]) * (BI[0] - o[0]) + (BI[1] - o[1]) * (BI[1] - o[1]) +
                            (BI[2] - o[2]) * (BI[2] - o[2]));
          if (dis > sqrt(2) * dx) {
            FWS[at(S, c, gi, gj, gk)] = IFLUID;
            continue;
          }
          /* surrounding cells of the image point in this cube */
          int ii, jj, kk, found = 0;
          for (ii = 0; ii <= nxx; ++ii) {
            double xc = Xcube[c] + (ii - 1.5) * dx;
            if (IP[0] >= xc && IP[0] <= xc + dx) { ++found; break; }
          }
          for (jj = 0; jj <= nxx; ++jj) {
            double yc = Ycube[c] + (jj - 1.5) * dx;
            if (IP[1] >= yc && IP[1] <= yc + dx) { ++found; break; }
          }
          for (kk = 0; kk <= nxx; ++kk) {
            double zc = Zcube[c] + (kk - 1.5) * dx;
            if (IP[2] >= zc && IP[2] <= zc + dx) { ++found; break; }
          }
          if (found < 3) continue;
          double xi = Xcube[c] + (ii - 1.5) * dx, yj = Ycube[c] + (jj - 1.5) * dx,
                 zk = Zcube[c] + (kk - 1.5) * dx;
          double s1 = IP[0] - xi, s2 = IP[1] - yj, s3 = IP[2] - zk;
          double hx = (Xcube[c] + (ii + 1 - 1.5) * dx) - xi;
          double hy = (Ycube[c] + (jj + 1 - 1.5) * dx) - yj;
          double hz = (Zcube[c] + (kk + 1 - 1.5) * dx) - zk;
          /* corners in the order 000, 100, 010, 001, 110, 101, 011, 111 */
          const int ox[8] = {0, 1, 0, 0, 1, 1, 0, 1}, oy[8] = {0, 0, 1, 0, 1, 0, 1, 1},
                    oz[8] = {0, 0, 0, 1, 0, 1, 1, 1};
          double V[64];
          for (int r = 0; r < 8; ++r) {
            double sx = ox[r] ? hx : 0, sy = oy[r] ? hy : 0, sz = oz[r] ? hz : 0;
            V[r * 8 + 7] = 1;
            V[r * 8 + 6] = sz;
            V[r * 8 + 5] = sy;
            V[r * 8 + 4] = sx;
            V[r * 8 + 3] = sy * sz;
            V[r * 8 + 2] = sx * sz;
            V[r * 8 + 1] = sx * sy;
            V[r * 8 + 0] = sx * sy * sz;
          }
          invert8(V);
          double w[8];
          int ok = 1;
          for (int r = 0; r < 8; ++r) {
            w[r] = V[r] * s1 * s2 * s3 + V[r + 8] * s1 * s2 + V[r + 16] * s1 * s3 +
                   V[r + 24] * s2 * s3 + V[r + 32] * s1 + V[r + 40] * s2 + V[r + 48] * s3 +
                   V[r + 56];
            if (!(w[r] >= (-MINIMUM) && w[r] <= (1 + MINIMUM))) ok = 0;
          }
          if (!ok) continue;
          int m = dotp >= 0 ? (*nminus)++ : (*nplus)++;
          if (m >= cap) return -1;
          int *G = dotp >= 0 ? gc_m : gc_p, *I = dotp >= 0 ? ip_m : ip_p;
          double *W = dotp >= 0 ? w_m : w_p;
          G[4 * m] = c; G[4 * m + 1] = gi; G[4 * m + 2] = gj; G[4 * m + 3] = gk;
          I[4 * m] = c; I[4 * m + 1] = ii; I[4 * m + 2] = jj; I[4 * m + 3] = kk;
          for (int r = 0; r < 8; ++r) W[8 * m + r] = w[r];
        }
  }
  return 0;
}
