/*
 * bcm_gb300 — GB300 (sm_103a) implementation of BCM_CGLI's per-cube
 * dual-time sub-iteration hot path, behind a C ABI.
 *
 * Two families of entry points:
 *
 *  1. Drop-in twins of the reference routines.  Same names, same parameter
 *     order and meaning, same in-place semantics on caller-owned host arrays
 *     in the reference layout U[Ncube][S][S][S][5] (S = NcubeX + 4),
 *     FWS[Ncube][S][S][S], 1-based cube numbering.  The reference fixes the
 *     resolution and prm.h constants at compile time; here they come from
 *     bcmg_set_reference_config() (defaults: the reference's Resolution.h and
 *     prm.h values).  Each call copies its arrays to the GPU, runs, and
 *     copies the results back.  They return void like the reference; a
 *     failure is reported by bcmg_last_error() (non-NULL after a failure).
 *
 *  2. A device-resident case context (bcmg_case_*): the state stays in HBM,
 *     one call advances whole dual-time steps (optionally replayed from a
 *     captured CUDA graph), and only the norms and snapshots cross to the
 *     host.
 *
 * All functions are thread-compatible, not thread-safe: one caller thread
 * per context (the reference is single-threaded at its call sites).
 */
#ifndef BCM_GB300_H
#define BCM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ----------------------------------------------------------------------- */
/* Status                                                                  */
/* ----------------------------------------------------------------------- */
#define BCMG_OK 0
#define BCMG_ERR_ARG 1        /* invalid argument / unsupported input */
#define BCMG_ERR_CUDA 2       /* CUDA runtime error */
#define BCMG_ERR_UNSUPPORTED 3 /* feature not available (e.g. multi-rank exchange) */

/* Last error message of the calling thread, or NULL if the last call on
 * this thread succeeded. */
const char *bcmg_last_error(void);

/* Library version string. */
const char *bcmg_version(void);

/* ----------------------------------------------------------------------- */
/* Reference compile-time configuration (Resolution.h / prm.h).            */
/* ----------------------------------------------------------------------- */
typedef struct bcmg_reference_config {
  int ncube_x;    /* NcubeX (Resolution.h:9); interior cells per cube edge */
  int mpi_ncube;  /* MPI_Ncube (Resolution.h:3); norm normaliser */
  double mu_L;    /* prm.h:5; 0 selects the inviscid kernel */
  double rho0;    /* prm.h:27 */
  double U0;      /* prm.h:29 */
  double Uin;     /* prm.h:31 */
  double P0;      /* prm.h:37 */
} bcmg_reference_config;

/* Sets the configuration the drop-in twins use; returns BCMG_OK. */
int bcmg_set_reference_config(const bcmg_reference_config *cfg);
void bcmg_get_reference_config(bcmg_reference_config *cfg);

/* Host arrays of the twins.  After bcmg_set_host_pinning(1) the twins
 * page-lock each caller array the first time they see it
 * (cudaHostRegister), so later copies run at the host link's full rate; an
 * array that cannot be registered is copied pageable.  Off by default: a
 * registration must end before its memory is freed, so only a caller whose
 * arrays outlive the calls (like the reference's main.cpp) should turn it
 * on, and it must call bcmg_release_host_arrays() (unregisters every array
 * and forgets it) before freeing any of them.  bcmg_set_host_pinning(0)
 * stops the page-locking and releases.
 *
 * BCM_Flux_XYZ_Viscous_Runge_kutta uploads the arrays a stage reads (RK 1:
 * U1_, U1, U1q; RK 2: also U1p1; RK 3: also U1p2 and Residual1, whose fluid
 * cells the norms sum) and, by default, also the ones it only writes, since
 * it returns them whole and writes only some of their cells.  With
 * bcmg_set_twin_scratch_kept(1) the write-only arrays (U1p1 at RK 1, U1p2 at
 * RK 2, Rku1, Residual1 at RK 1 and 2) are uploaded once per host array
 * instead: correct for a caller that, like the reference's main.cpp, keeps
 * those scratch arrays and changes them only through this routine (call
 * bcmg_release_host_arrays() when that stops being true). */
void bcmg_release_host_arrays(void);

/* Arithmetic of the BCM_Flux_XYZ_Viscous_Runge_kutta twin:
 * BCMG_PRECISION_FP64 (default, bit-identical to the reference) or
 * BCMG_PRECISION_SPLIT (FP32 reconstruction, fluxes, viscous terms and
 * preconditioner on deltas from the reference state, FP64 state update and
 * norms; within 1e-5 relative L2 of FP64, see the resident path).  With split
 * precision the stage update is applied inside the flux kernel, so Rku1 is
 * not written; U1_, U1p1 (RK 1), U1p2 (RK 2), Residual1 and er are.  Returns
 * BCMG_ERR_ARG for any other value. */
int bcmg_set_reference_precision(int precision);
void bcmg_set_host_pinning(int on);
void bcmg_set_twin_scratch_kept(int on);

/* ----------------------------------------------------------------------- */
/* 1. Drop-in twins of the reference routines                              */
/* ----------------------------------------------------------------------- */

/* Replaces BCM_Flux_XYZ_Viscous_Runge_kutta (main.h:473-513,
 * BCM_Flux_XYZ_Viscous_Runge_kutta.cpp:18-2659): one RK stage of residual,
 * pointwise-preconditioned increment and stage combination; at RK == 3 also
 * the change norms er[1..5] and force sums er[6..7].  Bit-identical to the
 * reference for U1_, U1p1, U1p2, Rku1 and Residual1.  csl is unused, as in
 * the reference. */
void BCM_Flux_XYZ_Viscous_Runge_kutta(int myid, int ncube, int RK, double deltaT,
                                      double deltaTau, double e, int *FWS, int *csl,
                                      double *cube_size, double *U1_, double *U1, double *U1q,
                                      double *U1p1, double *U1p2, double *Rku1,
                                      double *Residual1, double *er);

/* Replaces BCM_X_boundary_condition (main.h:418-434,
 * BCM_X_boundary_condition.cpp:19-122).  Xbc_l/Xbc_u are 1-based lists. */
void BCM_X_boundary_condition(int myid, int nXbc_l, int nXbc_u, int *Xbc_l, int *Xbc_u,
                              double *U1_);
/* Replaces BCM_Y_boundary_condition (main.h:439-451, BCM_Y_boundary_condition.cpp:17-89). */
void BCM_Y_boundary_condition(int nYbc_l, int nYbc_u, int *Ybc_l, int *Ybc_u, double *U1_);
/* Replaces BCM_Z_boundary_condition (main.h:459-470, BCM_Z_boundary_condition.cpp:20-96). */
void BCM_Z_boundary_condition(int nZbc_l, int nZbc_u, int *Zbc_l, int *Zbc_u, double *U1_);

/* Replace BCM_Ghostcell_minus / BCM_Ghostcell_plus (main.h:378-413,
 * BCM_Ghostcell_minus.cpp:17-495, BCM_Ghostcell_plus.cpp:16-489).  Tables
 * are the 1-based packed arrays of BCM_Reading_IBM.cpp:53-73; entries are
 * applied with the reference's serial-order semantics. */
void BCM_Ghostcell_minus(int myid, int *NNBC, double *weight, int *GCindex, int *IPsur,
                         int *FWS, double *U1_);
void BCM_Ghostcell_plus(int myid, int *NNBC, double *weight, int *GCindex, int *IPsur,
                        int *FWS, double *U1_);

/* Replaces BCM_Interface (main.h:224-354, BCM_Interface.cpp:27-5735) with
 * its full parameter list: same-level copies, 2:1 coarse/fine level jumps
 * (from the bs lists) and the ordered edge fill.  Single process: the
 * cross-rank exchange lists must be empty (ncpu_bs == ncpu_eq == ncpu_sb ==
 * 0), otherwise the call fails and leaves U1_ untouched. */
void BCM_Interface(int myid, int ncube, int mPI_Nadj, int ncpu_bs, int ncpu_eq, int ncpu_sb,
                   int max_nei_bs, int max_nei_eq, int max_nei_sb, int nadjX_eq, int nadjY_eq,
                   int nadjZ_eq, int nadjX_bs_plus, int nadjX_sb_plus, int nadjX_bs_minus,
                   int nadjX_sb_minus, int nadjY_bs_plus, int nadjY_sb_plus,
                   int nadjY_bs_minus, int nadjY_sb_minus, int nadjZ_bs_plus,
                   int nadjZ_sb_plus, int nadjZ_bs_minus, int nadjZ_sb_minus, int *rank_map,
                   int *MPI_cpu, int *MPI_cube, int *MPI_cpu_adj, int *MPI_cube_adj,
                   int *MPI_direction, int *MPI_interface, int *neighbor_cpu_eq,
                   int *Ncube_Ncpu_eq, int *neighbor_cpu_sb, int *Ncube_Ncpu_sb,
                   int *neighbor_cpu_bs, int *Ncube_Ncpu_bs, int *Scube_Ncpu_eq,
                   int *Rcube_Ncpu_eq, double *send_data_curr_eq, double *recv_data_curr_eq,
                   double *send_data_neig_eq, double *recv_data_neig_eq, int *Sdir_eq,
                   int *Rdir_eq, int *Scube_Ncpu_sb, int *Rcube_Ncpu_sb,
                   double *send_data_curr_sb, double *recv_data_curr_sb,
                   double *send_data_neig_sb, double *recv_data_neig_sb, int *Sdir_sb,
                   int *Rdir_sb, int *Scube_Ncpu_bs, int *Rcube_Ncpu_bs,
                   double *send_data_curr_bs, double *recv_data_curr_bs,
                   double *send_data_neig_bs, double *recv_data_neig_bs, int *Sdir_bs,
                   int *Rdir_bs, int *ist_eq, int *ist_sb, int *ist_bs, int *adjN_sb,
                   int *RadjN_bs, int *SadjN_bs, int *csl, int *adj_number, int *adjX_eq,
                   int *adjY_eq, int *adjZ_eq, int *adjX_bs_plus, int *adjX_sb_plus,
                   int *adjX_bs_minus, int *adjX_sb_minus, int *adjY_bs_plus,
                   int *adjY_sb_plus, int *adjY_bs_minus, int *adjY_sb_minus,
                   int *adjZ_bs_plus, int *adjZ_sb_plus, int *adjZ_bs_minus,
                   int *adjZ_sb_minus, double *U1_);

/* Replaces BCM_Immersed_boundary (main.h:113-144, BCM_Immersed_boundary.cpp
 * :127-1081; called once before the time loop, main.cpp:811).  Reads the
 * ASCII STL BCM_STL_fine.stl from the working directory, finds on the GPU
 * the boundary point, image point and trilinear weights of every IBM ghost
 * cell (FWS == 0) of the finest cubes, turns ghost cells farther than
 * sqrt(2) cells from the surface into fluid (FWS = 1) and writes
 * IBM_minus<myid>.dat / IBM_plus<myid>.dat byte for byte as the reference
 * does.  Cube resolution: bcmg_set_reference_config's ncube_x.  Xcnt, Ycnt,
 * Zcnt: cell centres [ncube][ncube_x+4] (NULL: formed from the corners).
 * n_wallcube, NBC, X/Y/Zmin/max and wallcube are accepted and unused, as in
 * the reference.  Errors (missing STL file, CUDA): bcmg_last_error(). */
void BCM_Immersed_boundary(int myid, int ncube, int n_wallcube, int *NBC, double Xmin,
                           double Xmax, double Ymin, double Ymax, double Zmin, double Zmax,
                           double *cube_size, int *csl, double *Xcube, double *Ycube,
                           double *Zcube, double *Xcnt, double *Ycnt, double *Zcnt, int *FWS,
                           int *wallcube);

/* Replaces BCM_FWS_Interface (main.h:55-110, BCM_FWS_Interface.cpp:23-791;
 * called at setup, main.cpp:634 and :1070).  In every finest-level cube
 * (csl == 0): the two ghost layers of each face with a same-level neighbour
 * take the neighbour's flags from the two interior layers beside the face
 * (pairs from the caller's 1-based lists adjX_eq / adjY_eq / adjZ_eq, the
 * neighbour read from slot 1 of adj_number), every flag becomes its sign,
 * and fluid or ghost cells with both neighbours along an axis solid become
 * solid until none is left (cells with every index in 1..ncube_x+2).  Other
 * cubes keep their flags.  Runs on the host (setup, integer work).  One
 * process: ncpu_eq must be 0; the other exchange arguments are accepted and
 * unused.  Errors (bad lists, pairs on different levels):
 * bcmg_last_error(), FWS unchanged. */
void BCM_FWS_Interface(int myid, int ncube, int mPI_Nadj, int ncpu_eq, int max_nei_eq,
                       int nadjX_eq, int nadjY_eq, int nadjZ_eq, int *rank_map, int *MPI_cpu,
                       int *MPI_cube, int *MPI_cpu_adj, int *MPI_cube_adj, int *MPI_direction,
                       int *MPI_interface, int *neighbor_cpu_eq, int *Ncube_Ncpu_eq,
                       int *Scube_Ncpu_eq, int *Rcube_Ncpu_eq, double *send_data_curr_eq,
                       double *recv_data_curr_eq, double *send_data_neig_eq,
                       double *recv_data_neig_eq, int *Sdir_eq, int *Rdir_eq, int *ist_eq,
                       int *csl, int *adj_number, int *adjX_eq, int *adjY_eq, int *adjZ_eq,
                       int *FWS);

/* The same for any cube edge n, with the same-level pairs found from
 * adj_number as BCM_Interface_table.cpp:96-120 classifies them.  FWS is
 * [ncube][n+4]^3.  Returns 0, or -1 for invalid input (bcmg_last_error()). */
int bcmg_fws_interface(int n, int ncube, const int *csl, const int *adj_number, int *FWS);

/* The same preprocessing in memory.  tri: ntri triangles x 3 vertices x
 * (x, y, z), in STL facet order.  Cell centres are formed from the cube
 * corners (BCM_Grid.cpp:124-148).  FWS ([ncube][n+4]^3) is updated in
 * place.  Tables (0-based arrays, up to `cap` entries each): gc_* = ghost
 * cell (cube, i, j, k), ip_* = the image point's base cell (cube, i, j, k),
 * w_* = eight weights, unrounded (the files hold them with six decimals);
 * minus = entries with dotp >= 0 (IBM_minus), plus = the others.  Returns
 * BCMG_ERR_ARG when an output table would exceed cap (FWS then untouched). */
int bcmg_ibm_preprocess(int n, int ncube, const double *cube_size, const int *csl,
                        const double *Xcube, const double *Ycube, const double *Zcube, int *FWS,
                        int ntri, const double *tri, int cap, int *nminus, int *gc_minus,
                        int *ip_minus, double *w_minus, int *nplus, int *gc_plus, int *ip_plus,
                        double *w_plus);

/* ----------------------------------------------------------------------- */
/* 2. Device-resident case context                                         */
/* ----------------------------------------------------------------------- */
#define BCMG_PRECISION_FP64 0  /* bit-exact with the reference */
#define BCMG_PRECISION_SPLIT 1 /* FP32 fluxes/preconditioner, FP64 state/source/norms */

typedef struct bcmg_case_desc {
  int n;          /* interior cells per cube edge */
  int ncube;      /* cube slots including the unused slot 0 (reference Ncube) */
  int mpi_ncube;  /* norm normaliser */
  double mu_L, rho0, U0, Uin, P0;
  double deltaT, deltaTau, e;
  int precision;  /* BCMG_PRECISION_* */
  const double *cube_size; /* [ncube] */
  const int *csl;          /* [ncube] */
  const int *adj_number;   /* [ncube][5][7] */
  const int *FWS;          /* [ncube][S][S][S] */
  /* Boundary-cube lists, 0-based arrays of cube numbers (main.cpp:147-189). */
  int nxl, nxu, nyl, nyu, nzl, nzu;
  const int *xl, *xu, *yl, *yu, *zl, *zu;
  /* IBM ghost tables, 1-based packed (BCM_Reading_IBM.cpp). */
  int nminus;
  const double *w_minus;
  const int *gc_minus, *ip_minus;
  int nplus;
  const double *w_plus;
  const int *gc_plus, *ip_plus;
} bcmg_case_desc;

typedef struct bcmg_case bcmg_case;

/* Creates a context on the current CUDA device and uploads geometry and
 * tables.  The state arrays are allocated and zeroed. */
int bcmg_case_create(const bcmg_case_desc *desc, bcmg_case **out);
void bcmg_case_destroy(bcmg_case *c);

/* Host <-> device state (full padded arrays, reference layout).  Any
 * pointer may be NULL to skip that array. */
int bcmg_case_set_state(bcmg_case *c, const double *U1_, const double *U1, const double *U1q);
int bcmg_case_get_state(bcmg_case *c, double *U1_, double *U1, double *U1q);
/* Scratch arrays as the reference keeps them (for parity checks). */
int bcmg_case_get_scratch(bcmg_case *c, double *U1p1, double *U1p2, double *Rku1,
                          double *Residual1);

/* One stage of the reference loop (main.cpp:1161-1241): BCs, IBM ghosts,
 * interface, flux/RK stage, interface. */
int bcmg_case_stage(bcmg_case *c, int RK);

/* `steps` dual-time steps of `subiters` sub-iterations each, followed by the
 * time-level shift (main.cpp:1146-1357).  use_graph != 0 captures one step
 * as a CUDA graph on first use and replays it.  er (8 doubles, 1-based like
 * the reference) and emax (6 doubles, E1..E5 at 1..5) are updated on the
 * host when non-NULL; emax carries the running maxima across calls. */
int bcmg_case_advance(bcmg_case *c, int steps, int subiters, int use_graph, double *er,
                      double *emax);

/* `steps` dual-time steps with the reference's convergence test
 * (main.cpp:1249-1271): each step sub-iterates until every normalised
 * change norm er[1..5] (E-normalised as in bcmg_case_advance) is below tol
 * (the reference uses 0.02) or max_subiters sub-iterations ran (the
 * reference's iteration_end_step), then shifts the time levels.  With
 * use_graph != 0 each step is one CUDA graph launch whose sub-iteration loop
 * is a device-side while node: no host round trip per sub-iteration.  In a
 * batch each case stops on its own test (the kernels skip converged cases),
 * so every case evolves as it would alone; the step ends when all cases
 * have.  subiters_out[step * ncase + q] receives the sub-iterations case q
 * took in each step (may be NULL); er and emax as in bcmg_case_advance. */
int bcmg_case_advance_converged(bcmg_case *c, int steps, int max_subiters, double tol,
                                int use_graph, int *subiters_out, double *er, double *emax);

/* PLOT3D output of BCM_Output (BCM_Output.cpp:16-300), byte-compatible:
 * raw native-endian files, header int32 ncube_out then (n+2, n+2, n+2) for
 * each of ncube_out cubes (the reference writes MPI_Ncube; <= 0 here means
 * the number of cubes written), then per cube the padded indices 1..n+2
 * with the first array index fastest.  Case q of a batch (q < 0: every cube
 * of the context).
 * bcmg_case_output_q writes the solution file (four 1.0 doubles and the
 * five variables of the current state U1_ per cube, main.cpp:1348)
 * asynchronously: it returns once the device snapshot is queued on the
 * context's stream, so solver calls may follow at once; the host copy and
 * the file write proceed on a side stream and a writer thread.
 * bcmg_case_output_wait waits for that write and returns its status (a
 * following output call or bcmg_case_destroy also waits).
 * bcmg_case_output_x writes the grid file synchronously: cell centres
 * origin + (i - 1.5) dx (BCM_Grid.cpp:124-148) from origin[ncube][3] (the
 * cube corners Xcube, Ycube, Zcube; rows of the case's own numbering, row 0
 * unused). */
int bcmg_case_output_q(bcmg_case *c, int q, int ncube_out, const char *path);
int bcmg_case_output_x(bcmg_case *c, int q, int ncube_out, const char *path,
                       const double *origin);
int bcmg_case_output_wait(bcmg_case *c);

/* Split-precision path: forms the FP32 mirror of the current state U1_ (the
 * deltas from each case's reference state (rho0, 0, 0, 0, P0/(K-1)) that the
 * flux kernel reads) and copies it to M[ncell][5] on the host, for checks. */
int bcmg_case_mirror(bcmg_case *c, float *M);
/* The mirror as the kernels keep it during stepping (the current buffer,
 * not re-formed), for checks: it equals the rounding of the current state
 * in every cell. */
int bcmg_case_mirror_current(bcmg_case *c, float *M);

/* Launch shapes.  flux_tile: edge of the cube tile one flux CTA works on,
 * 8 or 4 (0: 8 when it divides n, else 4); flux_form (split precision, 8^3
 * tiles): 1 each thread evaluates its two faces of an axis together in
 * packed FP32 pairs (Blackwell FFMA2/FADD2/FMUL2), 2 one after the other, 0
 * the default (1); lusgs_threads: threads per cube of the split-precision
 * LU-SGS sweep, a multiple of 32 up to the widest plane of a cube (0: the
 * widest plane; fewer threads take wide planes in several passes).  The
 * shapes change how work is spread over the GPU, not the FP64 path's
 * arithmetic (it stays bit-identical to the reference); the two split flux
 * forms round differently (both within the split path's error bound).
 * bcmg_case_autotune times the candidates on the context's own state with
 * CUDA events (`reps` launches each, state restored), applies the fastest
 * and reports every time in `out` (flux_ms: tile 8 packed, tile 8 one face
 * at a time, tile 4; lusgs_ms: widest plane, half of it; 0 where not
 * measured).  The LU-SGS candidates are timed only on the split path with
 * LU-SGS selected. */
typedef struct bcmg_tuning {
  int flux_tile;
  int lusgs_threads;
  int flux_form;
  double flux_ms[3];
  double lusgs_ms[2];
} bcmg_tuning;
int bcmg_case_set_tuning(bcmg_case *c, const bcmg_tuning *t);
int bcmg_case_autotune(bcmg_case *c, int reps, bcmg_tuning *out);

/* Where split-precision RK stages and LU-SGS sweeps make the interface's
 * same-level face copies of the updated cells: in_flux = 1 (default) inside
 * the updating kernel, each updated cell next to a same-level face writing
 * its new value into the neighbour's ghost layer, so the interface call
 * after the update runs only the level-jump tasks and the edge fill; 0: in
 * that interface call.  Both give the same bits.  No effect on the FP64
 * path. */
int bcmg_case_set_face_copies(bcmg_case *c, int in_flux);

/* Split-precision path: how the FP32 mirror of the state (the deltas the
 * flux and LU-SGS kernels read) is kept.  on = 0 (default): formed whole
 * once per dual-time step (and per bcmg_case_stage call); within the step
 * every kernel that writes the state writes the mirror values of the cells
 * it writes (the flux kernel into a second buffer, since other blocks read
 * its cells' old values during the launch).  on = 1: formed whole before
 * every flux launch instead (a pass over every cell; for checks).  Both
 * give the same bits.  No effect on the FP64 path. */
int bcmg_case_set_mirror_each_stage(bcmg_case *c, int on);

/* The IBM ghost-cell fill of each stage on a second stream, beside the
 * boundary fill, with the interface call after them waiting for both.  In
 * effect (the default) for every case (of a batch) in which no IBM entry's
 * cell (ghost cell or stencil) lies in the three layers the boundary fill
 * touches at a boundary face of its cube, so the two fills touch disjoint
 * cells; the other cases' entries, and all of them with on = 0, are filled
 * after the boundary fill in the reference's order.  Both give the same
 * bits.  bcmg_case_concurrent_ghosts returns 1 where some entries are
 * filled beside the boundary fill. */
int bcmg_case_set_concurrent_ghosts(bcmg_case *c, int on);
int bcmg_case_concurrent_ghosts(bcmg_case *c);

/* Asynchronous stepping, for pipelines that overlap host transfers of one
 * context with the steps of another: bcmg_case_advance_async enqueues
 * `steps` graph launches of a step of `subiters` sub-iterations on the
 * context's stream and returns (the first call for a sub-iteration count
 * captures the graph and waits for that; not with profiling or an exchange
 * hook); bcmg_case_copy_state_async enqueues the copies of the non-NULL
 * arrays between the host and the device (to_device != 0: host -> device;
 * page-locked host memory makes them asynchronous; the host arrays must stay
 * untouched until bcmg_case_sync); bcmg_case_get_norms waits for the stream
 * and copies er / emax (as bcmg_case_advance would return them). */
int bcmg_case_advance_async(bcmg_case *c, int steps, int subiters);
int bcmg_case_copy_state_async(bcmg_case *c, int to_device, double *U1_, double *U1,
                               double *U1q);
int bcmg_case_get_norms(bcmg_case *c, double *er, double *emax);

/* Waits for all work of the context. */
int bcmg_case_sync(bcmg_case *c);

/* Device pointers of the state arrays (for zero-copy use by the caller). */
int bcmg_case_device_state(bcmg_case *c, double **U1_, double **U1, double **U1q);

/* Number of kernel launches issued by the last bcmg_case_advance call
 * (counted on the host, graph replays count their nodes). */
long long bcmg_case_launch_count(const bcmg_case *c);

/* Times `reps` launches of the flux kernel alone on the current state with
 * CUDA events on the context's stream; returns the average milliseconds per
 * launch in *ms (the launch covers every cube once, RK stage 1 arithmetic,
 * increments only: the state is not modified). */
int bcmg_case_time_flux(bcmg_case *c, int reps, double *ms);

/* Per-launch timing of the flux kernel inside bcmg_case_advance: with
 * profiling on, CUDA events on the context's stream bracket every flux
 * launch (graphs are not used while profiling).  bcmg_case_profile returns
 * the accumulated milliseconds and launch count since profiling was
 * (re)enabled. */
int bcmg_case_set_profiling(bcmg_case *c, int on);
int bcmg_case_profile(const bcmg_case *c, double *flux_ms_total, long long *flux_launches);

/* Batch of independent cases in one context.  No counterpart in the
 * reference, which runs one case per process: here the cases (same n and
 * precision; any cube counts, constants, time steps, boundaries and IBM
 * tables) are laid end to end in one flat cube list, so each stage is the
 * same launches as for one case, over all cubes of all cases.  Case q's
 * cube l becomes cube cube0_q + l - 1 (bcmg_case_case_cubes); every other
 * bcmg_case_* call works on the whole batch, and bcmg_case_advance's er and
 * emax become [ncase][8] and [ncase][6] (per case, each with its own
 * normalisers).  Each case's state evolves exactly as it would in a context
 * of its own. */
int bcmg_batch_create(int ncase, const bcmg_case_desc *descs, bcmg_case **out);

/* Sub-iteration method of bcmg_case_advance.  BCMG_METHOD_RK3 (default) is
 * the reference's three-stage preconditioned RK (bit-exact).  BCMG_METHOD_LUSGS
 * has no counterpart in the reference (BCM_LUSGS.h there holds no solver):
 * one matrix-free LU-SGS step per sub-iteration for the same residual
 * (split Jacobians with relaxation omega in [1, 4], scalar viscous term, a
 * local pseudo-time term when cfl > 0, none when cfl == 0), swept per cube
 * over the planes i+j+k = const.  It converges to the state the RK
 * sub-iterations converge to, in fewer sub-iterations; er and emax keep
 * their meaning (change norms of each update).  On the split-precision
 * path the sweeps run in FP32 on the FP32 mirror of the state, the update
 * and norm sums in FP64. */
#define BCMG_METHOD_RK3 0
#define BCMG_METHOD_LUSGS 1
int bcmg_case_set_method(bcmg_case *c, int method, double cfl, double omega);
int bcmg_case_ncase(const bcmg_case *c);
/* First flat cube of case q and the case's own cube-slot count (ncube of
 * its descriptor, unused slot 0 included). */
int bcmg_case_case_cubes(const bcmg_case *c, int q, int *cube0, int *ncube);
/* State of case q in its own layout [ncube_q][S][S][S][5] (slot 0 ignored);
 * any pointer may be NULL. */
int bcmg_case_set_case_state(bcmg_case *c, int q, const double *U1_, const double *U1,
                             const double *U1q);
int bcmg_case_get_case_state(bcmg_case *c, int q, double *U1_, double *U1, double *U1q);

/* One FP64 RK stage that allocates nothing.  No counterpart in the
 * reference.  It serves callers that cannot let a library call cudaMalloc:
 * solvers that hand out every device buffer from their own pre-sized arena,
 * and latency-sensitive hosts that cannot accept the implicit device
 * synchronisation an allocation may cause.  Same arithmetic as
 * BCM_Flux_XYZ_Viscous_Runge_kutta (with the bcmg_set_reference_config
 * values): U1_, U1p1, U1p2, Rku1 and Residual1 are bit-identical to it; the
 * norms er[1..7] are summed over fixed 4096-cell blocks, a different order,
 * so they agree within rounding (about 1e-12 relative).  Unlike it, every
 * array argument is a DEVICE pointer owned by the caller
 * (cube_size and er included; er[0] is set to 0), the work is queued on
 * `stream` (a cudaStream_t, NULL for the legacy default stream) and the call
 * returns without waiting.  Its only scratch, the per-block norm partial
 * sums, is a fixed static device array (8192 blocks x 7 doubles, 458 KB)
 * that every GPU loading the library holds until the process exits; cases
 * above 33,554,432 interior cells are rejected with BCMG_ERR_ARG.  The first
 * call on a device looks up that array's device address (once per device,
 * with that device current); make that first call before any stream
 * capture.  Every call shares the scratch, and each call fully rewrites the
 * part it reads, so nothing needs clearing; calls that overlap on the GPU
 * (other streams, other host threads) race on it and must be serialised by
 * the caller. */
int bcmg_flux_rk_stage_noalloc(int ncube, int RK, double deltaT, double deltaTau, double e,
                               const int *FWS, const double *cube_size, double *U1_,
                               const double *U1, const double *U1q, double *U1p1,
                               double *U1p2, double *Rku1, double *Residual1, double *er,
                               void *stream);

/* Cube-sharded runs (one rank per GPU).  The reference spreads cubes over
 * MPI ranks by rank_map.dat (main.cpp:576-596), exchanges the face layers
 * of cubes on other ranks in every interface call (BCM_Interface.cpp
 * :213-1738, :4367-5634) and sums the norms with MPI_Allreduce
 * (BCM_Flux_XYZ_Viscous_Runge_kutta.cpp:2641-2652).  Here a rank's context
 * holds its own cubes in slots 1..nlocal and, after them, nproxy "proxy"
 * slots: remote cubes whose faces its cubes' face tasks read.  Proxies are
 * never advanced; before every interface call the exchange hook must fill
 * the proxies' face bands (bcmg_case_halo_pack on the owning rank, the
 * transport of the caller's choice, bcmg_case_halo_unpack here), and after
 * the norm sums of a sub-iteration it must replace the 7 raw sums
 * (bcmg_case_norm_sums) by their sum over the ranks.  The cells then evolve
 * bit for bit as in one context holding every cube.
 *
 * bcmg_shard_plan: the cubes of rank `rank` (local_cubes, ascending) and the
 * remote cubes its face tasks read (proxy_cubes, ascending), global numbers;
 * rank_of_cube[ncube] (slot 0 unused).  bcmg_shard_bands: the face bands
 * rank dst_rank reads from rank src_rank, 4 ints each (global source cube,
 * axis 0..2, side 1 high / 0 low face of the source, interior layers next to
 * it: 2, or 4 for fine -> coarse averages), in one fixed order, so the
 * sender and the receiver compute the same list.  Both return 0, -1 for
 * invalid input, -2 when a list exceeds cap (the counts are still set). */
int bcmg_shard_plan(int ncube, const int *adj_number, const int *csl, const int *rank_of_cube,
                    int rank, int cap, int *nlocal, int *local_cubes, int *nproxy,
                    int *proxy_cubes);
int bcmg_shard_bands(int ncube, const int *adj_number, const int *csl, const int *rank_of_cube,
                     int src_rank, int dst_rank, int cap, int *nband, int *bands);

/* Flags of a sharded run at setup (the cross-rank part of
 * BCM_FWS_Interface.cpp:136-550): the owning rank packs the flag bands of
 * its cubes (4 ints per band in local slots: cube, axis, side, layers, as
 * for bcmg_case_set_halo; layers * n * n ints per band in (layer, first
 * in-face index, second) order), the receiving rank unpacks them into its
 * proxy slots and then calls bcmg_fws_interface on its own cubes and
 * proxies: its cubes' flags equal those of one process holding the whole
 * case.  Host memory; 0, or -1 for invalid input. */
int bcmg_fws_band_pack(int n, int ncube, const int *FWS, int nband, const int *bands, int *buf);
int bcmg_fws_band_unpack(int n, int ncube, int *FWS, int nband, const int *bands,
                         const int *buf);

/* A rank's context: desc describes its nlocal + nproxy cubes in local
 * numbering (cube slot 1 + i: local_cubes[i], then proxy_cubes) with the
 * adjacency mapped to local slots (entries naming a cube of neither list:
 * 0), boundary lists and IBM tables of its own cubes only.  Face tasks into
 * proxies are dropped; tasks out of proxies run in every interface call.
 * Batches are not sharded. */
int bcmg_case_create_shard(const bcmg_case_desc *desc, int nproxy, bcmg_case **out);

/* Exchange hook, called in the context's stream order (stream = the
 * context's cudaStream_t) with phase BCMG_XCHG_HALO before every interface
 * call and BCMG_XCHG_NORMS after the norm sums of a sub-iteration; returns
 * 0, or non-zero to fail the stepping call.  A context with a hook steps
 * without CUDA graphs (use_graph must be 0). */
#define BCMG_XCHG_HALO 0
#define BCMG_XCHG_NORMS 1
typedef int (*bcmg_exchange_fn)(void *user, int phase, void *stream);
int bcmg_case_set_exchange(bcmg_case *c, bcmg_exchange_fn fn, void *user);

/* Halo bands per peer, in local cube slots: send[p] (4 ints per band: a
 * local cube 1..nlocal, axis, side, layers) are packed for peer p, recv[p]
 * (a proxy slot) unpacked from it, each in the order bcmg_shard_bands gives.
 * bcmg_case_halo_bytes: buffer bytes of one peer's send / recv (every
 * cell's five doubles, plus five floats on the split path).  pack / unpack
 * enqueue on the context's stream; dev_buf is device memory of at least
 * those bytes. */
int bcmg_case_set_halo(bcmg_case *c, int npeer, const int *nsend, const int *const *send,
                       const int *nrecv, const int *const *recv);
int bcmg_case_halo_bytes(const bcmg_case *c, int peer, size_t *send_bytes, size_t *recv_bytes);
int bcmg_case_halo_pack(bcmg_case *c, int peer, void *dev_buf);
int bcmg_case_halo_unpack(bcmg_case *c, int peer, const void *dev_buf);
/* Device address of the 7 raw norm sums (squared changes of p, u, v, w, T
 * and the two force sums) that the BCMG_XCHG_NORMS hook adds over the ranks
 * in place. */
int bcmg_case_norm_sums(bcmg_case *c, double **dev_sums);
/* The same 7 sums through host memory (for a host-side transport): write =
 * 0 copies them to sums[7], write = 1 copies sums[7] back; both wait for the
 * copy. */
int bcmg_case_norm_sums_host(bcmg_case *c, double *sums, int write);

/* Device-time marks on the context's stream: bcmg_case_timer_mark records
 * event `slot` (0..15); bcmg_case_timer_elapsed waits for mark b and returns
 * the milliseconds between marks a and b. */
int bcmg_case_timer_mark(bcmg_case *c, int slot);
int bcmg_case_timer_elapsed(bcmg_case *c, int a, int b, double *ms);

/* Measured FP64 fused-multiply-add rate of the current device in GFLOP/s
 * (2 flops per FMA), from a short dependent-chain kernel: the ALU roof for
 * the FP64 path. */
int bcmg_probe_fp64_rate(double *gflops);

/* ----------------------------------------------------------------------- */
/* Host-side table builders (no GPU needed)                                */
/* ----------------------------------------------------------------------- */

/* Dependency levels of an IBM ghost table (1-based packed GCindex/IPsur of
 * nbc entries, cube resolution n, ncube slots).  Entries of one level are
 * independent; applying levels 1, 2, ... reproduces the reference's serial
 * loop (BCM_Ghostcell_minus.cpp:72).  level_of_entry[e-1] receives entry e's
 * level.  Returns the number of levels, or -1 for invalid input (an index
 * outside the case's arrays). */
int bcmg_ibm_schedule(int nbc, const int *GCindex, const int *IPsur, int n, int ncube,
                      int *level_of_entry);

/* Interface copy tasks derived from adj_number/csl like
 * BCM_Interface_table.cpp:96-308: task_off[ncube+1] (CSR by destination
 * cube) and task_words[5*t..] = (source cube, axis 0..2, side 0 low / 1 high
 * ghost layers, kind 0 same-level / 1 coarse->fine / 2 fine->coarse, sub-face
 * slot 1..4 for kinds 1 and 2).  Returns the task count, -1 for invalid input
 * (out-of-range adjacency, a jump larger than 2:1, inconsistent faces), -2
 * if max_tasks is too small. */
int bcmg_interface_tasks(int ncube, const int *adj_number, const int *csl, int *task_off,
                         int *task_words, int max_tasks);

/* The interface plan of a resident context, for the tasks of
 * bcmg_interface_tasks (same order).  keep_prologue[t] = 1 when the
 * interface call ahead of a stage must repeat task t right after the
 * previous stage's closing call (level jumps; faces the boundary fill
 * writes, from the 0-based boundary lists as in bcmg_case_desc; faces whose
 * ghost or source layers hold an IBM ghost cell, from the 1-based GC
 * tables).  push[6 ncube]: the split flux kernel's same-level push table
 * (push[6 c + 2 axis + 0]: cube whose high ghost layers copy cube c's
 * layers 2, 3; + 1: cube whose low ghost layers copy layers n, n+1; 0 where
 * none).  Returns the task count, -1 for invalid input, -2 if max_tasks is
 * too small, -3 if a push slot would need two destinations (the context
 * then keeps the copies in the interface call). */
int bcmg_interface_plan(int n, int ncube, const int *adj_number, const int *csl,
                        const int *const bc_lists[6], const int bc_counts[6],
                        const int *gc_minus, int nminus, const int *gc_plus, int nplus,
                        int *keep_prologue, int *push, int max_tasks);

/* The reduced closing interface call of split-precision RK stages 1 and 2
 * in a resident context, for the tasks of bcmg_interface_tasks (same order):
 * keep_closing[t] = 1 for the level-jump tasks whose ghost face is read
 * before the next stage's opening call rewrites it (by the boundary fill's
 * y and z faces, or by an IBM stencil reaching into its cube's ghost
 * layers; IP tables 1-based), edge_cubes[c] = 1 (c < ncube) for the cubes
 * whose edge fill such a read sees.  Returns the task count, -1 for invalid
 * input, -2 if max_tasks is too small. */
/* Per case of a resident context (case_cube0: each case's first cube, then
 * one past the last; {1, ncube} for one case): beside[q] = 1 when the
 * case's IBM ghost fill may run beside the boundary fill, i.e. none of its
 * entries' cells (ghost cell, stencil) lies in the three layers the boundary
 * fill touches at a boundary face of its cube, no stencil lies in another
 * case, and the context has boundary faces.  Boundary lists 0-based as in
 * bcmg_case_desc, GC / IP tables 1-based.  Returns ncase, -1 for invalid
 * input. */
int bcmg_ghost_beside_plan(int n, int ncube, const int *const bc_lists[6], const int bc_counts[6],
                           const int *gc_minus, const int *ip_minus, int nminus,
                           const int *gc_plus, const int *ip_plus, int nplus,
                           const int *case_cube0, int ncase, int *beside);

int bcmg_interface_closing_plan(int n, int ncube, const int *adj_number, const int *csl,
                                const int *const bc_lists[6], const int bc_counts[6],
                                const int *ip_minus, int nminus, const int *ip_plus, int nplus,
                                int *keep_closing, int *edge_cubes, int max_tasks);

#ifdef __cplusplus
}
#endif
#endif
