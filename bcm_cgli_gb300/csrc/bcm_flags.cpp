// The flag field's same-level interface (BCM_FWS_Interface.cpp:23-791), on
// the host.  The reference calls it twice per run, at setup (main.cpp:634,
// after the grid is read, and main.cpp:1070, after the IBM preprocessing has
// turned some ghost cells fluid), over integer flags, before any solver
// work; the flags then go to the device with the case.
//
// What the routine leaves behind on one rank:
//  1. In every finest-level cube (csl == 0), each ghost face cell (the two
//     ghost layers of a face, over the face's n x n interior) next to a
//     same-level neighbour holds the neighbour's flag from the two interior
//     layers beside the face (:555-660), for the same-level pairs of
//     BCM_Interface_table.cpp:96-120 (X, then Y, then Z; each list in cube
//     order).  The copies read interior cells only and write ghost cells
//     only, so they are made in place; where two pairs write one face the
//     later pair wins, as in the reference's serial order.
//  2. Every cell of a finest-level cube is replaced by its sign: the
//     reference copies the flags into doubles and thresholds them at +-0.5
//     (:668-700), which for integers is the sign.
//  3. Holes (:702-783): a fluid or ghost cell (flag >= 0) with every index in
//     1..n+2 whose two neighbours along some axis are both solid becomes
//     solid, until no cell changes.  The rule only ever turns cells solid,
//     and a solid neighbour can only make it hold, so the cells that end
//     solid are the smallest set closed under the rule, whatever the order
//     of visits: the reference sweeps the cube in memory order until a sweep
//     fills nothing; here a work list re-examines the neighbours of each
//     newly filled cell only.
// Cubes of other levels keep their flags.
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "bcm_flags.h"
#include "bcm_trace.h"

namespace bcmg {
namespace {

constexpr int kSolid = -1;

struct Cube {
  int *f;
  int S;
  int &at(int i, int j, int k) const { return f[((size_t)i * S + j) * S + k]; }
};

// In-face coordinates of a face along axis ax: the other two axes, x<y<z.
inline void face_axes(int ax, int *t0, int *t1) {
  *t0 = ax == 0 ? 1 : 0;
  *t1 = ax == 2 ? 1 : 2;
}

// Cube c2 (the +axis neighbour of c): its low ghost layers take c's layers
// n, n+1; c's high ghost layers take c2's layers 2, 3.
void copy_pair(int n, int *F, int c, int c2, int ax) {
  const int S = n + 4;
  const size_t per = (size_t)S * S * S;
  const Cube A{F + per * c, S}, B{F + per * c2, S};
  int t0, t1;
  face_axes(ax, &t0, &t1);
  for (int l = 0; l < 2; ++l)
    for (int p = 2; p <= n + 1; ++p)
      for (int q = 2; q <= n + 1; ++q) {
        int lo[3], hi[3], ia[3], ib[3];
        lo[t0] = hi[t0] = ia[t0] = ib[t0] = p;
        lo[t1] = hi[t1] = ia[t1] = ib[t1] = q;
        lo[ax] = l;          // c2's low ghost layer l
        ia[ax] = n + l;      // from c's layer n + l
        hi[ax] = n + 2 + l;  // c's high ghost layer n + 2 + l
        ib[ax] = 2 + l;      // from c2's layer 2 + l
        B.at(lo[0], lo[1], lo[2]) = A.at(ia[0], ia[1], ia[2]);
        A.at(hi[0], hi[1], hi[2]) = B.at(ib[0], ib[1], ib[2]);
      }
}

void fill_holes(int n, int *f) {
  const int S = n + 4, lo = 1, hi = n + 2;
  const Cube C{f, S};
  auto hole = [&](int i, int j, int k) {
    if (C.at(i, j, k) < 0) return false;
    return (C.at(i + 1, j, k) == kSolid && C.at(i - 1, j, k) == kSolid) ||
           (C.at(i, j + 1, k) == kSolid && C.at(i, j - 1, k) == kSolid) ||
           (C.at(i, j, k + 1) == kSolid && C.at(i, j, k - 1) == kSolid);
  };
  std::vector<int> work;
  for (int i = lo; i <= hi; ++i)
    for (int j = lo; j <= hi; ++j)
      for (int k = lo; k <= hi; ++k)
        if (hole(i, j, k)) work.push_back((i * S + j) * S + k);
  while (!work.empty()) {
    const int w = work.back();
    work.pop_back();
    const int i = w / (S * S), j = (w / S) % S, k = w % S;
    if (!hole(i, j, k)) continue;  // filled already, or not (yet) a hole
    C.at(i, j, k) = kSolid;
    const int nb[6][3] = {{i - 1, j, k}, {i + 1, j, k}, {i, j - 1, k},
                          {i, j + 1, k}, {i, j, k - 1}, {i, j, k + 1}};
    for (const auto &x : nb)
      if (x[0] >= lo && x[0] <= hi && x[1] >= lo && x[1] <= hi && x[2] >= lo && x[2] <= hi &&
          C.at(x[0], x[1], x[2]) >= 0)
        work.push_back((x[0] * S + x[1]) * S + x[2]);
  }
}

std::string msg(const char *f, long long a, long long b = 0) {
  char buf[200];
  std::snprintf(buf, sizeof buf, f, a, b);
  return buf;
}

}  // namespace

bool same_level_pairs(int ncube, const int *adj, const int *csl, std::vector<int> pairs[3],
                      std::string &err) {
  auto A = [&](int c, int s, int d) { return adj[(c * 5 + s) * 7 + d]; };
  for (int ax = 0; ax < 3; ++ax) {
    pairs[ax].clear();
    const int dir = 2 + 2 * ax;
    for (int c = 1; c < ncube; ++c) {
      int any = 0, acube = 0;
      for (int s = 1; s <= 4; ++s) {
        const int a = A(c, s, dir);
        if (a < 0 || a >= ncube) {
          err = msg("flag interface: cube %lld: neighbour %lld out of range", c, a);
          return false;
        }
        any |= a > 0;
        acube = std::max(acube, a);
      }
      if (any && csl[c] == csl[acube]) pairs[ax].push_back(c);
    }
  }
  return true;
}

bool fws_interface(int n, int ncube, const int *csl, const int *adj,
                   const std::vector<int> pairs[3], int *FWS, std::string &err) {
  if (n < 1 || ncube < 1 || !csl || !adj || !FWS) {
    err = "flag interface: bad arguments";
    return false;
  }
  for (int ax = 0; ax < 3; ++ax)
    for (int c : pairs[ax]) {
      const int c2 = c > 0 && c < ncube ? adj[(c * 5 + 1) * 7 + 2 + 2 * ax] : -1;
      if (c <= 0 || c >= ncube || c2 <= 0 || c2 >= ncube) {
        err = msg("flag interface: same-level pair of cube %lld on axis %lld has no neighbour",
                  c, ax);
        return false;
      }
      if (csl[c] != csl[c2]) {
        err = msg("flag interface: cubes %lld and %lld of a same-level pair differ in level",
                  c, c2);
        return false;
      }
    }
  const int S = n + 4;
  const size_t per = (size_t)S * S * S;
  for (int ax = 0; ax < 3; ++ax)
    for (int c : pairs[ax])
      if (csl[c] == 0) copy_pair(n, FWS, c, adj[(c * 5 + 1) * 7 + 2 + 2 * ax], ax);
  for (int c = 1; c < ncube; ++c) {
    if (csl[c] != 0) continue;
    int *f = FWS + per * c;
    for (size_t x = 0; x < per; ++x) f[x] = (f[x] > 0) - (f[x] < 0);
    fill_holes(n, f);
  }
  return true;
}

bool fws_bands(int n, int ncube, int *FWS, int nband, const int *bands, int *buf, bool unpack,
               std::string &err) {
  if (n < 1 || ncube < 1 || nband < 0 || (nband > 0 && (!FWS || !bands || !buf))) {
    err = "flag bands: bad arguments";
    return false;
  }
  for (int b = 0; b < nband; ++b) {
    const int c = bands[4 * b], ax = bands[4 * b + 1], side = bands[4 * b + 2],
              L = bands[4 * b + 3];
    if (c < 1 || c >= ncube || ax < 0 || ax > 2 || side < 0 || side > 1 || L < 1 || L > n) {
      err = msg("flag bands: band %lld invalid (cube %lld)", b, c);
      return false;
    }
  }
  const int S = n + 4;
  size_t h = 0;
  for (int b = 0; b < nband; ++b) {
    const int c = bands[4 * b], ax = bands[4 * b + 1], side = bands[4 * b + 2],
              L = bands[4 * b + 3];
    const Cube C{FWS + (size_t)S * S * S * c, S};
    int t0, t1;
    face_axes(ax, &t0, &t1);
    const int l0 = side == 1 ? n + 2 - L : 2;
    for (int l = 0; l < L; ++l)
      for (int p = 0; p < n; ++p)
        for (int q = 0; q < n; ++q, ++h) {
          int x[3];
          x[ax] = l0 + l;
          x[t0] = 2 + p;
          x[t1] = 2 + q;
          int &v = C.at(x[0], x[1], x[2]);
          if (unpack)
            v = buf[h];
          else
            buf[h] = v;
        }
  }
  return true;
}

}  // namespace bcmg

// ---------------------------------------------------------------------------
// C entry points.
// ---------------------------------------------------------------------------
#include "../../include/bcm_gb300.h"

extern "C" void bcmg_internal_set_error(const char *msg);

extern "C" int bcmg_fws_interface(int n, int ncube, const int *csl, const int *adj_number,
                                  int *FWS) {
  std::vector<int> pairs[3];
  std::string err;
  if (n < 1 || ncube < 1 || !csl || !adj_number || !FWS ||
      !bcmg::same_level_pairs(ncube, adj_number, csl, pairs, err) ||
      !bcmg::fws_interface(n, ncube, csl, adj_number, pairs, FWS, err)) {
    bcmg_internal_set_error(err.empty() ? "bcmg_fws_interface: bad arguments" : err.c_str());
    return -1;
  }
  return 0;
}

extern "C" int bcmg_fws_band_pack(int n, int ncube, const int *FWS, int nband,
                                  const int *bands, int *buf) {
  std::string err;
  if (!bcmg::fws_bands(n, ncube, const_cast<int *>(FWS), nband, bands, buf, false, err)) {
    bcmg_internal_set_error(err.c_str());
    return -1;
  }
  return 0;
}

extern "C" int bcmg_fws_band_unpack(int n, int ncube, int *FWS, int nband, const int *bands,
                                    const int *buf) {
  std::string err;
  if (!bcmg::fws_bands(n, ncube, FWS, nband, bands, const_cast<int *>(buf), true, err)) {
    bcmg_internal_set_error(err.c_str());
    return -1;
  }
  return 0;
}

// Drop-in twin of BCM_FWS_Interface (main.h:55-110, BCM_FWS_Interface.cpp
// :23-791), parameters in the reference's order, cube edge from
// bcmg_set_reference_config.  One rank: non-empty cross-rank lists
// (ncpu_eq > 0) are rejected (a sharded run packs and unpacks flag bands
// with bcmg_fws_band_pack / bcmg_fws_band_unpack instead); the same-level
// pairs are the caller's lists adjX_eq / adjY_eq / adjZ_eq (1-based, as
// BCM_Interface_table builds them).  Failures leave FWS unchanged and are
// reported by bcmg_last_error().
extern "C" void BCM_FWS_Interface(int myid, int ncube, int mPI_Nadj, int ncpu_eq,
                                  int max_nei_eq, int nadjX_eq, int nadjY_eq, int nadjZ_eq,
                                  int *rank_map, int *MPI_cpu, int *MPI_cube, int *MPI_cpu_adj,
                                  int *MPI_cube_adj, int *MPI_direction, int *MPI_interface,
                                  int *neighbor_cpu_eq, int *Ncube_Ncpu_eq,
                                  int *Scube_Ncpu_eq, int *Rcube_Ncpu_eq,
                                  double *send_data_curr_eq, double *recv_data_curr_eq,
                                  double *send_data_neig_eq, double *recv_data_neig_eq,
                                  int *Sdir_eq, int *Rdir_eq, int *ist_eq, int *csl,
                                  int *adj_number, int *adjX_eq, int *adjY_eq, int *adjZ_eq,
                                  int *FWS) {
  bcmg::TraceRange trace("BCM_FWS_Interface");
  (void)myid; (void)mPI_Nadj; (void)max_nei_eq; (void)rank_map; (void)MPI_cpu; (void)MPI_cube;
  (void)MPI_cpu_adj; (void)MPI_cube_adj; (void)MPI_direction; (void)MPI_interface;
  (void)neighbor_cpu_eq; (void)Ncube_Ncpu_eq; (void)Scube_Ncpu_eq; (void)Rcube_Ncpu_eq;
  (void)send_data_curr_eq; (void)recv_data_curr_eq; (void)send_data_neig_eq;
  (void)recv_data_neig_eq; (void)Sdir_eq; (void)Rdir_eq; (void)ist_eq;
  bcmg_internal_set_error(nullptr);
  if (ncpu_eq) {
    bcmg_internal_set_error("BCM_FWS_Interface: cross-rank exchange lists are not supported "
                            "in one process (use bcmg_fws_band_pack / _unpack)");
    return;
  }
  bcmg_reference_config cfg;
  bcmg_get_reference_config(&cfg);
  const int counts[3] = {nadjX_eq, nadjY_eq, nadjZ_eq};
  const int *lists[3] = {adjX_eq, adjY_eq, adjZ_eq};
  bool bad = ncube < 1 || !csl || !adj_number || !FWS;
  for (int a = 0; a < 3; ++a) bad |= counts[a] < 0 || (counts[a] > 0 && !lists[a]);
  if (bad) {
    bcmg_internal_set_error("BCM_FWS_Interface: bad arguments");
    return;
  }
  std::vector<int> pairs[3];
  for (int a = 0; a < 3; ++a) pairs[a].assign(lists[a] + (counts[a] ? 1 : 0),
                                              lists[a] + (counts[a] ? counts[a] + 1 : 0));
  std::string err;
  if (!bcmg::fws_interface(cfg.ncube_x, ncube, csl, adj_number, pairs, FWS, err))
    bcmg_internal_set_error(("BCM_FWS_Interface: " + err).c_str());
}
