/*
 * Test-infrastructure driver around the reference's OWN compiled sources.
 *
 * It is compiled together with the reference's BCM_*.cpp files (taken from
 * where they lie, never copied) by oracle/ref_build.py, against a generated
 * per-configuration Resolution.h / prm.h and the single-rank MPI stub in
 * oracle/mpi_stub.  It only forwards arrays to the reference routines and
 * replays the per-stage call order of the reference time loop
 * (main.cpp:1146-1357), so the reference itself is the thing executed.
 * Nothing here is part of the product.
 */
#include <stdlib.h>
#include <string.h>
#include <omp.h>
#include "main.h"

int Ncube = 0;
int N_wallcube = 1;
int MPI_Nadj = 1;
int Max_nei_eq = 0, Max_nei_sb = 0, Max_nei_bs = 0;
int Ncpu_eq = 0, Ncpu_sb = 0, Ncpu_bs = 0;
int NBC_minus = 0, NBC_plus = 0, NBC = 0;
int NXbc_l = 0, NXbc_u = 0, NYbc_l = 0, NYbc_u = 0, NZbc_l = 0, NZbc_u = 0;

typedef double Cell[X_size][Y_size][Z_size][Ndim];
typedef int Flag[X_size][Y_size][Z_size];

namespace {

/* Interface tables as built by the reference's BCM_Interface_table. */
struct Tables {
  int ncube = 0;
  int *csl = nullptr;
  int (*adj)[5][7] = nullptr;
  int n[15];
  int *lists[15];
};
Tables T;

/* Dummy single-rank MPI bookkeeping: every exchange list is empty. */
struct MpiLists {
  int one[4] = {0, 0, 0, 0};
  double dz[4] = {0, 0, 0, 0};
  int (*rank_map)[MPI_Ncube] = nullptr;
};
MpiLists M;

void free_tables() {
  for (int l = 0; l < 15; ++l) { free(T.lists[l]); T.lists[l] = nullptr; }
  free(T.csl); T.csl = nullptr;
  free(T.adj); T.adj = nullptr;
}

}  // namespace

extern "C" {

int ref_x_size(void) { return X_size; }
int ref_ncube_x(void) { return NcubeX; }
int ref_mpi_ncube(void) { return MPI_Ncube; }
void ref_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }

/* BCM_Flux_XYZ_Viscous_Runge_kutta (main.h:473-513), one RK stage. */
void ref_flux(int ncube, int RK, double dT, double dTau, double e, int *FWS, int *csl,
              double *cube_size, double *U1_, double *U1, double *U1q, double *U1p1,
              double *U1p2, double *Rku1, double *Residual1, double *er) {
  Ncube = ncube;
  BCM_Flux_XYZ_Viscous_Runge_kutta(0, ncube, RK, dT, dTau, e, (Flag *)FWS, csl, cube_size,
                                   (Cell *)U1_, (Cell *)U1, (Cell *)U1q, (Cell *)U1p1,
                                   (Cell *)U1p2, (Cell *)Rku1, (Cell *)Residual1, er);
}

/* BCM_X/Y/Z_boundary_condition in the order of main.cpp:1161-1165. */
void ref_bc(int nxl, int nxu, int *xl, int *xu, int nyl, int nyu, int *yl, int *yu, int nzl,
            int nzu, int *zl, int *zu, double *U1_) {
  NXbc_l = nxl; NXbc_u = nxu; NYbc_l = nyl; NYbc_u = nyu; NZbc_l = nzl; NZbc_u = nzu;
  BCM_X_boundary_condition(0, nxl, nxu, xl, xu, (Cell *)U1_);
  BCM_Y_boundary_condition(nyl, nyu, yl, yu, (Cell *)U1_);
  BCM_Z_boundary_condition(nzl, nzu, zl, zu, (Cell *)U1_);
}

/* BCM_Ghostcell_minus (which < 0) or BCM_Ghostcell_plus (which > 0). */
void ref_ghost(int which, int n, double *weight, int *GCindex, int *IPsur, int *FWS,
               double *U1_) {
  int nn = n;
  if (which < 0) {
    NBC_minus = n;
    BCM_Ghostcell_minus(0, &nn, weight, GCindex, IPsur, (Flag *)FWS, (Cell *)U1_);
  } else {
    NBC_plus = n;
    BCM_Ghostcell_plus(0, &nn, weight, GCindex, IPsur, (Flag *)FWS, (Cell *)U1_);
  }
}

/* Build the interface lists with the reference's BCM_Interface_table.
 * adj_number is [ncube][5][7], csl is [ncube]; both 1-based like the reference.
 * Writes the 15 list lengths to counts (order: X eq, X bs+, X sb+, X bs-, X sb-,
 * then Y, then Z) when counts is non-null. */
void ref_interface_setup(int ncube, const int *adj_number, const int *csl, int *counts) {
  free_tables();
  Ncube = ncube;
  T.ncube = ncube;
  T.csl = (int *)malloc(sizeof(int) * (size_t)ncube);
  memcpy(T.csl, csl, sizeof(int) * (size_t)ncube);
  T.adj = (int(*)[5][7])malloc(sizeof(int) * 35 * (size_t)ncube);
  memcpy(T.adj, adj_number, sizeof(int) * 35 * (size_t)ncube);
  for (int l = 0; l < 15; ++l) T.lists[l] = (int *)calloc((size_t)ncube + 1, sizeof(int));
  int *n = T.n;
  BCM_Interface_table(0, ncube, N_wallcube, &n[0], &n[5], &n[10], &n[1], &n[2], &n[3], &n[4],
                      &n[6], &n[7], &n[8], &n[9], &n[11], &n[12], &n[13], &n[14], T.csl,
                      T.adj, T.lists[0], T.lists[5], T.lists[10], T.lists[1], T.lists[2],
                      T.lists[3], T.lists[4], T.lists[6], T.lists[7], T.lists[8], T.lists[9],
                      T.lists[11], T.lists[12], T.lists[13], T.lists[14]);
  if (counts)
    for (int l = 0; l < 15; ++l) counts[l] = n[l];
  if (!M.rank_map) M.rank_map = (int(*)[MPI_Ncube])calloc(2 * (size_t)MPI_Ncube, sizeof(int));
}

/* Copy list l (1-based entries 1..n[l]) into out. */
void ref_interface_list(int l, int *out) {
  for (int a = 1; a <= T.n[l]; ++a) out[a - 1] = T.lists[l][a];
}

/* BCM_Interface (main.h:224-354) with the tables from ref_interface_setup and
 * empty single-rank exchange lists. */
void ref_interface(double *U1_) {
  int *z = M.one;
  double *d = M.dz;
  int *n = T.n;
  int **L = T.lists;
  BCM_Interface(0, T.ncube, MPI_Nadj, 0, 0, 0, 0, 0, 0, n[0], n[5], n[10], n[1], n[2], n[3],
                n[4], n[6], n[7], n[8], n[9], n[11], n[12], n[13], n[14], M.rank_map, z, z, z,
                z, z, z, z, z, z, z, z, z, z, z, d, d, d, d, z, z, z, z, d, d, d, d, z, z, z, z,
                d, d, d, d, z, z, z, z, z, z, z, z, T.csl, T.adj, L[0], L[5], L[10], L[1], L[2],
                L[3], L[4], L[6], L[7], L[8], L[9], L[11], L[12], L[13], L[14], (Cell *)U1_);
}

/* BCM_FWS_Interface (main.h:55-110) with the same-level lists from
 * ref_interface_setup and empty single-rank exchange lists; FWS is
 * [ncube][X_size]^3, changed in place. */
void ref_fws_interface(int *FWS) {
  int *z = M.one;
  double *d = M.dz;
  int *n = T.n;
  BCM_FWS_Interface(0, T.ncube, MPI_Nadj, 0, 0, n[0], n[5], n[10], M.rank_map, z, z, z, z, z,
                    z, z, z, z, z, d, d, d, d, z, z, z, T.csl, T.adj, T.lists[0], T.lists[5],
                    T.lists[10], (Flag *)FWS);
}

/*
 * The reference time loop (main.cpp:1146-1357) for `steps` physical steps of
 * exactly `subiters` pseudo-time sub-iterations each (the reference's own loop
 * stops at iteration_end_step; a fixed count keeps runs comparable).
 * Per stage: BCs X,Y,Z -> IBM ghost minus, plus -> interface -> flux/RK ->
 * interface.  After the last sub-iteration of a step: time-level shift
 * U1q <- U1, U1 <- U1_ on interior cells.  er[8] receives the last stage-3
 * norms (after the E-normalisation of main.cpp:1249-1259) and Emax[6] the
 * running maxima E1..E5 (index 1..5).
 */
void ref_run(int ncube, int steps, int subiters, double dT, double dTau, double e, int *FWS,
             int *csl, double *cube_size, double *U1_, double *U1, double *U1q, double *U1p1,
             double *U1p2, double *Rku1, double *Residual1, int nxl, int nxu, int *xl, int *xu,
             int nyl, int nyu, int *yl, int *yu, int nzl, int nzu, int *zl, int *zu,
             int nminus, double *wm, int *gm, int *im, int nplus, double *wp, int *gp, int *ip,
             double *er, double *Emax) {
  Cell *u_ = (Cell *)U1_, *u = (Cell *)U1, *uq = (Cell *)U1q;
  for (int step = 1; step <= steps; ++step) {
    for (int it = 1; it <= subiters; ++it) {
      for (int RK = 1; RK < 4; ++RK) {
        ref_bc(nxl, nxu, xl, xu, nyl, nyu, yl, yu, nzl, nzu, zl, zu, U1_);
        if (nminus > 0) ref_ghost(-1, nminus, wm, gm, im, FWS, U1_);
        if (nplus > 0) ref_ghost(1, nplus, wp, gp, ip, FWS, U1_);
        ref_interface(U1_);
        ref_flux(ncube, RK, dT, dTau, e, FWS, csl, cube_size, U1_, U1, U1q, U1p1, U1p2, Rku1,
                 Residual1, er);
        ref_interface(U1_);
      }
      for (int v = 1; v <= 5; ++v) {
        Emax[v] = er[v] > Emax[v] ? er[v] : Emax[v];
        er[v] = er[v] / Emax[v];
      }
    }
    for (int c = 1; c < ncube; ++c)
      for (int i = n_buffer; i <= nx; ++i)
        for (int j = n_buffer; j <= ny; ++j)
          for (int k = n_buffer; k <= nz; ++k)
            for (int v = 0; v < Ndim; ++v) {
              uq[c][i][j][k][v] = u[c][i][j][k][v];
              u[c][i][j][k][v] = u_[c][i][j][k][v];
            }
  }
}

/* BCM_Output (BCM_Output.cpp:16-300) on one rank: the PLOT3D grid file
 * BCMdata00001.x and solution file qBCMdata<step>.q of U1 in the current
 * directory.  Cell-centre coordinates as BCM_Grid.cpp:124-148 forms them
 * from the cube origins. */
void ref_output(int ncube, int step, double *U1, double *cube_size, const double *Xcube,
                const double *Ycube, const double *Zcube) {
  Ncube = ncube;
  int (*rank_map)[MPI_Ncube] = (int (*)[MPI_Ncube])calloc(2 * (size_t)MPI_Ncube, sizeof(int));
  double (*Xcnt)[X_size] = (double (*)[X_size])calloc((size_t)ncube * X_size, sizeof(double));
  double (*Ycnt)[Y_size] = (double (*)[Y_size])calloc((size_t)ncube * Y_size, sizeof(double));
  double (*Zcnt)[Z_size] = (double (*)[Z_size])calloc((size_t)ncube * Z_size, sizeof(double));
  for (int c = 1; c < ncube; ++c) {
    double dx = cube_size[c] / NcubeX, dy = cube_size[c] / NcubeY, dz = cube_size[c] / NcubeZ;
    for (int i = 0; i < X_size; ++i) Xcnt[c][i] = Xcube[c] + (i - 1.5) * dx;
    for (int j = 0; j < Y_size; ++j) Ycnt[c][j] = Ycube[c] + (j - 1.5) * dy;
    for (int k = 0; k < Z_size; ++k) Zcnt[c][k] = Zcube[c] + (k - 1.5) * dz;
  }
  BCM_Output(0, ncube, step, rank_map, (Cell *)U1, (Cell *)U1, cube_size, Xcnt, Ycnt, Zcnt);
  free(rank_map);
  free(Xcnt);
  free(Ycnt);
  free(Zcnt);
}

/* BCM_Immersed_boundary (BCM_Immersed_boundary.cpp:127-1081) on one rank:
 * reads BCM_STL_fine.stl and writes IBM_minus00000.dat / IBM_plus00000.dat
 * in the current directory; FWS is updated in place (ghost cells whose
 * boundary point lies too far become fluid).  Cell centres as
 * BCM_Grid.cpp:124-148 forms them. */
void ref_ibm(int ncube, double *cube_size, int *csl, double *Xcube, double *Ycube,
             double *Zcube, int *FWS) {
  Ncube = ncube;
  double (*Xcnt)[X_size] = (double (*)[X_size])calloc((size_t)ncube * X_size, sizeof(double));
  double (*Ycnt)[Y_size] = (double (*)[Y_size])calloc((size_t)ncube * Y_size, sizeof(double));
  double (*Zcnt)[Z_size] = (double (*)[Z_size])calloc((size_t)ncube * Z_size, sizeof(double));
  for (int c = 1; c < ncube; ++c) {
    double dx = cube_size[c] / NcubeX, dy = cube_size[c] / NcubeY, dz = cube_size[c] / NcubeZ;
    for (int i = 0; i < X_size; ++i) Xcnt[c][i] = Xcube[c] + (i - 1.5) * dx;
    for (int j = 0; j < Y_size; ++j) Ycnt[c][j] = Ycube[c] + (j - 1.5) * dy;
    for (int k = 0; k < Z_size; ++k) Zcnt[c][k] = Zcube[c] + (k - 1.5) * dz;
  }
  int NBC = 0;
  int wallcube[2] = {0, 0};
  BCM_Immersed_boundary(0, ncube, 1, &NBC, 0., 0., 0., 0., 0., 0., cube_size, csl, Xcube, Ycube,
                        Zcube, Xcnt, Ycnt, Zcnt, (Flag *)FWS, wallcube);
  free(Xcnt);
  free(Ycnt);
  free(Zcnt);
}

}  // extern "C"
