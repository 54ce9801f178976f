// Host-side table builders: they turn the reference's setup data (adjacency,
// boundary-cube lists, IBM ghost tables) into conflict-free launch tables
// for the GPU kernels, validating every index on the way so no kernel can
// address memory outside the case's arrays.
#include "bcm_tables.h"

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstdio>
#include <map>
#include <unordered_map>

namespace bcmg {

static std::string fmt(const char *f, long long a = 0, long long b = 0, long long c = 0) {
  char buf[256];
  std::snprintf(buf, sizeof buf, f, a, b, c);
  return buf;
}

namespace {

// Collects face tasks in the reference's order (BCM_Interface.cpp: per axis
// same-level copies, then blocks (a), (b), (c), (d) of the level jumps) and
// keeps the last writer of each destination face (or face quadrant), which is
// what the reference's serial loops leave behind.
struct TaskSet {
  int ncube;
  // key: dst cube, axis, side -> whole-face writer (kind 0/1) or quadrant
  // writers (kind 2, slots 1..4)
  std::vector<FaceTask> whole;     // [ncube*6]
  std::vector<FaceTask> quad;      // [ncube*6*4]
  std::vector<char> has_whole, has_quad;
  explicit TaskSet(int nc)
      : ncube(nc), whole((size_t)nc * 6), quad((size_t)nc * 24), has_whole((size_t)nc * 6, 0),
        has_quad((size_t)nc * 24, 0) {}
  void put(int dst, int src, int ax, int side, int kind, int slot) {
    FaceTask t;
    t.src = src;
    t.axis = (int8_t)ax;
    t.side = (int8_t)side;
    t.kind = (int8_t)kind;
    t.slot = (int8_t)slot;
    const size_t f = (size_t)dst * 6 + ax * 2 + side;
    if (kind == 2) {
      quad[f * 4 + (slot - 1)] = t;
      has_quad[f * 4 + (slot - 1)] = 1;
    } else {
      whole[f] = t;
      has_whole[f] = 1;
    }
  }
  bool finish(std::vector<int> &off, std::vector<FaceTask> &tasks, std::string &err) {
    off.assign((size_t)ncube + 1, 0);
    tasks.clear();
    for (int c = 0; c < ncube; ++c) {
      off[c] = (int)tasks.size();
      if (c == 0) continue;
      for (int fs = 0; fs < 6; ++fs) {
        const size_t f = (size_t)c * 6 + fs;
        bool anyq = false;
        for (int q = 0; q < 4; ++q) anyq |= has_quad[f * 4 + q] != 0;
        if (has_whole[f] && anyq) {
          err = fmt("cube %lld: one face is both a whole-face and a sub-face destination "
                    "(inconsistent adjacency)", c);
          return false;
        }
        if (has_whole[f]) tasks.push_back(whole[f]);
        for (int q = 0; q < 4; ++q)
          if (has_quad[f * 4 + q]) tasks.push_back(quad[f * 4 + q]);
      }
    }
    off[ncube] = (int)tasks.size();
    return true;
  }
};

bool check_adj(int ncube, const int *adj, std::string &err) {
  for (int c = 1; c < ncube; ++c)
    for (int s = 1; s <= 4; ++s)
      for (int d = 1; d <= 6; ++d) {
        int v = adj[(c * 5 + s) * 7 + d];
        if (v < 0 || v >= ncube) {
          err = fmt("adj_number[%lld][%lld][*] out of range", c, s);
          return false;
        }
      }
  return true;
}

// Tasks of the four level-jump blocks of one big cube B on axis ax; pm 0:
// its +ax neighbours are the small cubes, pm 1: its -ax neighbours.
void level_tasks(TaskSet &T, const int *adj, int B, int ax, int pm, bool inject) {
  const int dir = pm == 0 ? 2 + 2 * ax : 1 + 2 * ax;
  for (int sl = 1; sl <= 4; ++sl) {
    const int sc = adj[(B * 5 + sl) * 7 + dir];
    if (sc <= 0) continue;
    if (inject)
      T.put(sc, B, ax, pm == 0 ? 0 : 1, 1, sl);  // (a) / (b): small's ghosts facing B
    else
      T.put(B, sc, ax, pm == 0 ? 1 : 0, 2, sl);  // (c) / (d): B's quadrant
  }
}

}  // namespace

// Face tasks from adjacency, classifying neighbours like
// BCM_Interface_table.cpp:96-308: a cube has a +dir (-dir) relation when any
// of the four slots adj_number[c][1..4][dir] is positive; the classifying
// cube is the largest slot value; same level when csl matches, big->small
// when this cube's csl is larger.  The same-level copy partner is slot 1
// (:1753).  Level jumps must be 2:1.
bool build_interface_tasks(int ncube, const int *adj, const int *csl, std::vector<int> &off,
                           std::vector<FaceTask> &tasks, std::string &err) {
  if (!check_adj(ncube, adj, err)) return false;
  auto A = [&](int c, int s, int d) { return adj[(c * 5 + s) * 7 + d]; };
  TaskSet T(ncube);
  for (int ax = 0; ax < 3; ++ax) {
    std::vector<int> bsp, bsm;
    for (int c = 1; c < ncube; ++c) {
      for (int pm = 0; pm < 2; ++pm) {
        const int dir = pm == 0 ? 2 + 2 * ax : 1 + 2 * ax;
        int any = 0, acube = 0;
        for (int s = 1; s <= 4; ++s) {
          any |= A(c, s, dir) > 0;
          acube = std::max(acube, A(c, s, dir));
        }
        if (!any) continue;
        const int dl = csl[c] - csl[acube];
        if (dl > 1 || dl < -1) {
          err = fmt("cube %lld: level jump larger than 2:1 on axis %lld", c, ax);
          return false;
        }
        if (pm == 0 && dl == 0) {
          const int c2 = A(c, 1, dir);
          if (c2 <= 0) {
            err = fmt("cube %lld: +axis %lld neighbour missing from slot 1", c, ax);
            return false;
          }
          T.put(c2, c, ax, 0, 0, 0);  // c2 low ghosts <- c high interior
          T.put(c, c2, ax, 1, 0, 0);  // c high ghosts <- c2 low interior
        }
        if (dl == 1) (pm == 0 ? bsp : bsm).push_back(c);
      }
    }
    for (int B : bsp) level_tasks(T, adj, B, ax, 0, true);
    for (int B : bsm) level_tasks(T, adj, B, ax, 1, true);
    for (int B : bsp) level_tasks(T, adj, B, ax, 0, false);
    for (int B : bsm) level_tasks(T, adj, B, ax, 1, false);
  }
  return T.finish(off, tasks, err);
}

// The same tasks from explicit reference lists (adjX_eq, adjX_bs_plus,
// adjX_bs_minus, ... 1-based with counts), as BCM_Interface receives them.
bool build_interface_tasks_from_lists(int ncube, const int *adj, const int *csl,
                                      const int *const lists[9], const int counts[9],
                                      std::vector<int> &off, std::vector<FaceTask> &tasks,
                                      std::string &err) {
  (void)csl;
  if (!check_adj(ncube, adj, err)) return false;
  TaskSet T(ncube);
  for (int ax = 0; ax < 3; ++ax) {
    for (int l = 0; l < 3; ++l)
      for (int a = 1; a <= counts[3 * ax + l]; ++a) {
        const int c = lists[3 * ax + l][a];
        if (c <= 0 || c >= ncube) {
          err = fmt("interface list %lld entry %lld out of range", 3 * ax + l, a);
          return false;
        }
      }
    const int dplus = 2 + 2 * ax;
    for (int a = 1; a <= counts[3 * ax]; ++a) {
      const int c = lists[3 * ax][a];
      const int c2 = adj[(c * 5 + 1) * 7 + dplus];
      if (c2 <= 0) {
        err = fmt("cube %lld: neighbour on axis %lld missing", c, ax);
        return false;
      }
      T.put(c2, c, ax, 0, 0, 0);
      T.put(c, c2, ax, 1, 0, 0);
    }
    for (int a = 1; a <= counts[3 * ax + 1]; ++a) level_tasks(T, adj, lists[3 * ax + 1][a], ax, 0, true);
    for (int a = 1; a <= counts[3 * ax + 2]; ++a) level_tasks(T, adj, lists[3 * ax + 2][a], ax, 1, true);
    for (int a = 1; a <= counts[3 * ax + 1]; ++a) level_tasks(T, adj, lists[3 * ax + 1][a], ax, 0, false);
    for (int a = 1; a <= counts[3 * ax + 2]; ++a) level_tasks(T, adj, lists[3 * ax + 2][a], ax, 1, false);
  }
  return T.finish(off, tasks, err);
}

bool build_bc_entries(int ncube, const int *const lists[6], const int counts[6],
                      std::vector<int> &cubes, std::vector<int> &masks, std::string &err) {
  std::vector<int> m((size_t)ncube, 0);
  for (int l = 0; l < 6; ++l)
    for (int a = 0; a < counts[l]; ++a) {
      int c = lists[l][a];
      if (c <= 0 || c >= ncube) {
        err = fmt("boundary list %lld entry %lld out of range", l, a);
        return false;
      }
      m[c] |= 1 << l;
    }
  cubes.clear();
  masks.clear();
  for (int c = 1; c < ncube; ++c)
    if (m[c]) {
      cubes.push_back(c);
      masks.push_back(m[c]);
    }
  return true;
}

// Dependency levels for the IBM ghost entries (BCM_Ghostcell_minus.cpp:72).
// The reference applies entries serially; an entry may read a ghost another
// entry writes.  Level(e) = 1 + the highest level among earlier entries
// that write a cell e reads (read-after-write), read the cell e writes
// (write-after-read) or write the same cell (write-after-write).  Entries of
// one level touch disjoint written cells and read no cell written in that
// level, so a level can run fully parallel and the sequence of levels
// reproduces the serial result exactly.
bool build_ibm_levels(int nbc, const int *GC, const int *IP, int n, int ncube,
                      std::vector<int> &order, std::vector<int> &level_off, std::string &err) {
  const int S = n + 4;
  struct Tag {
    int write = 0;  // level of the last writer
    int read = 0;   // highest level of any reader so far
  };
  std::unordered_map<long long, Tag> cells;
  cells.reserve((size_t)nbc * 9 + 16);
  std::vector<int> lev((size_t)nbc + 1, 0);
  int maxlev = 0;
  auto key = [&](int c, int i, int j, int k) {
    return (((long long)c * S + i) * S + j) * S + k;
  };
  for (int e = 1; e <= nbc; ++e) {
    const int b = (e - 1) * 4;
    const int c = IP[b + 1], i = IP[b + 2], j = IP[b + 3], k = IP[b + 4];
    const int gc = GC[b + 1], gi = GC[b + 2], gj = GC[b + 3], gk = GC[b + 4];
    if (c <= 0 || c >= ncube || i < 0 || j < 0 || k < 0 || i + 1 >= S || j + 1 >= S ||
        k + 1 >= S) {
      err = fmt("IBM entry %lld: image-point stencil out of range", e);
      return false;
    }
    if (gc <= 0 || gc >= ncube || gi < 0 || gj < 0 || gk < 0 || gi >= S || gj >= S || gk >= S) {
      err = fmt("IBM entry %lld: ghost cell out of range", e);
      return false;
    }
    int L = 1;
    for (int m = 0; m < 8; ++m) {
      auto it = cells.find(key(c, i + (m & 1), j + ((m >> 1) & 1), k + ((m >> 2) & 1)));
      if (it != cells.end()) L = std::max(L, it->second.write + 1);
    }
    const long long w = key(gc, gi, gj, gk);
    auto it = cells.find(w);
    if (it != cells.end()) L = std::max(L, std::max(it->second.read, it->second.write) + 1);
    lev[e] = L;
    maxlev = std::max(maxlev, L);
    for (int m = 0; m < 8; ++m) {
      Tag &t = cells[key(c, i + (m & 1), j + ((m >> 1) & 1), k + ((m >> 2) & 1))];
      t.read = std::max(t.read, L);
    }
    cells[w].write = L;
  }
  level_off.assign((size_t)maxlev + 1, 0);
  for (int e = 1; e <= nbc; ++e) level_off[lev[e]]++;
  // prefix: level_off[l-1]..level_off[l] holds level l (levels 1..maxlev)
  std::vector<int> start((size_t)maxlev + 2, 0);
  for (int l = 1; l <= maxlev; ++l) start[l + 1] = start[l] + level_off[l];
  order.assign((size_t)nbc, 0);
  std::vector<int> fill(start.begin(), start.end());
  for (int e = 1; e <= nbc; ++e) order[fill[lev[e]]++] = e;
  level_off.assign((size_t)maxlev + 1, 0);
  for (int l = 0; l <= maxlev; ++l) level_off[l] = start[l + 1];
  return true;
}

void prologue_task_mask(int n, int ncube, const std::vector<FaceTask> &tasks,
                        const std::vector<int> &task_cube, const std::vector<int> &bc_cubes,
                        const std::vector<int> &bc_masks, const int *gc_minus, int nminus,
                        const int *gc_plus, int nplus, std::vector<char> &keep) {
  // Per cube, bits 0..5: ghost face (axis, side) written by the boundary
  // fill or holding an IBM ghost cell; bits 6..11: the interior layers a
  // neighbour's face (axis, side) copies from hold an IBM ghost cell.
  std::vector<uint16_t> hot((size_t)std::max(ncube, 0), 0);
  for (size_t q = 0; q < bc_cubes.size(); ++q) hot[bc_cubes[q]] |= (uint16_t)(bc_masks[q] & 63);
  auto mark = [&](const int *G, int cnt) {
    for (int e = 0; e < cnt; ++e) {
      const int g = G[1 + 4 * e];
      const int x[3] = {G[2 + 4 * e], G[3 + 4 * e], G[4 + 4 * e]};
      if (g <= 0 || g >= ncube) continue;
      for (int ax = 0; ax < 3; ++ax) {
        const int a = x[(ax + 1) % 3], b = x[(ax + 2) % 3];
        if (a < 2 || a > n + 1 || b < 2 || b > n + 1) continue;
        const int l = x[ax];
        if (l == 0 || l == 1) hot[g] |= (uint16_t)(1 << (2 * ax));
        if (l == n + 2 || l == n + 3) hot[g] |= (uint16_t)(1 << (2 * ax + 1));
        if (l == n || l == n + 1) hot[g] |= (uint16_t)(1 << (6 + 2 * ax));
        if (l == 2 || l == 3) hot[g] |= (uint16_t)(1 << (6 + 2 * ax + 1));
      }
    }
  };
  if (gc_minus && nminus > 0) mark(gc_minus, nminus);
  if (gc_plus && nplus > 0) mark(gc_plus, nplus);
  keep.assign(tasks.size(), 0);
  for (size_t t = 0; t < tasks.size(); ++t) {
    const FaceTask &f = tasks[t];
    const int face = 2 * f.axis + f.side;
    keep[t] = f.kind != 0 || (hot[task_cube[t]] >> face & 1) || (hot[f.src] >> (6 + face) & 1);
  }
}

// The closing interface call of RK stages 1 and 2 on the split path (the
// level jumps and the edge fill after the update).  The next stage's opening
// call runs every level jump and the edge fill again, so of the closing
// call's writes only those read before it matter: the boundary fill's y
// faces read the x-ghost rows of their cube (all i, j = 2 or n + 1), its z
// faces the x- and y-ghost rows and the edge cells (all i, j, k = 2 or
// n + 1), and an IBM stencil may reach into its cube's ghost layers (face
// ghosts, or edge cells where two coordinates are ghost).  keep[t] for the
// tasks of the closing list (level jumps) writing such a face; edge[c] for
// the cubes whose edge fill such a read sees.
void closing_plan(int n, int ncube, const std::vector<FaceTask> &tasks,
                  const std::vector<int> &task_cube, const std::vector<int> &bc_cubes,
                  const std::vector<int> &bc_masks, const int *ip_minus, int nminus,
                  const int *ip_plus, int nplus, std::vector<char> &keep,
                  std::vector<char> &edge) {
  std::vector<uint8_t> face((size_t)std::max(ncube, 0), 0);  // bit 2 axis + side
  edge.assign((size_t)std::max(ncube, 0), 0);
  for (size_t q = 0; q < bc_cubes.size(); ++q) {
    const int c = bc_cubes[q], m = bc_masks[q];
    if (c <= 0 || c >= ncube) continue;
    if (m & 12) face[c] |= 3;  // y faces read the x ghost rows
    if (m & 48) {              // z faces: x and y ghost rows, edge cells
      face[c] |= 15;
      edge[c] = 1;
    }
  }
  auto ghost_side = [&](int x) { return x <= 1 ? 0 : (x >= n + 2 ? 1 : -1); };
  auto mark = [&](const int *I, int cnt) {
    for (int e = 0; e < cnt; ++e) {
      const int c = I[1 + 4 * e];
      if (c <= 0 || c >= ncube) continue;
      for (int d = 0; d < 8; ++d) {
        const int x[3] = {I[2 + 4 * e] + (d & 1), I[3 + 4 * e] + (d >> 1 & 1),
                          I[4 + 4 * e] + (d >> 2 & 1)};
        int ghosts = 0;
        for (int ax = 0; ax < 3; ++ax) {
          const int sd = ghost_side(x[ax]);
          if (sd < 0) continue;
          ++ghosts;
          face[c] |= (uint8_t)(1 << (2 * ax + sd));
        }
        if (ghosts >= 2) edge[c] = 1;
      }
    }
  };
  if (ip_minus && nminus > 0) mark(ip_minus, nminus);
  if (ip_plus && nplus > 0) mark(ip_plus, nplus);
  keep.assign(tasks.size(), 0);
  for (size_t t = 0; t < tasks.size(); ++t) {
    const FaceTask &f = tasks[t];
    keep[t] = f.kind != 0 && (face[task_cube[t]] >> (2 * f.axis + f.side) & 1);
  }
}

// The cases whose IBM ghost fill must follow the boundary fill: some entry's
// cell (ghost cell or one of its eight stencil cells) lies in the three
// layers the boundary fill touches at a boundary face of its cube (ghost
// layers written, the next interior layer read; y and z faces over whole
// planes), or its stencil lies in another case.  The other cases' entries
// touch no cell the boundary fill reads or writes.  GC/IP 1-based, ne
// entries; case_cube0[q] is case q's first cube (ncase + 1 values; a single
// case: {1, ncube}).
void ghost_shared_cases(int n, int ncube, const std::vector<int> &bc_cubes,
                        const std::vector<int> &bc_masks, const int *GC, const int *IP, int ne,
                        const std::vector<int> &case_cube0, std::vector<char> &shared) {
  const int ncs = (int)case_cube0.size() - 1;
  shared.assign((size_t)std::max(ncs, 0), 0);
  auto case_of = [&](int cube) -> int {
    return (int)(std::upper_bound(case_cube0.begin(), case_cube0.end(), cube) -
                 case_cube0.begin()) - 1;
  };
  std::vector<int> bcmask((size_t)std::max(ncube, 0), 0);
  for (size_t q = 0; q < bc_cubes.size(); ++q)
    if (bc_cubes[q] > 0 && bc_cubes[q] < ncube) bcmask[bc_cubes[q]] |= bc_masks[q];
  auto in_slab = [&](int cube, int i, int j, int k) {
    if (cube <= 0 || cube >= ncube) return true;
    const int m = bcmask[cube], x[3] = {i, j, k};
    for (int ax = 0; ax < 3; ++ax) {
      if ((m >> (2 * ax) & 1) && x[ax] <= 2) return true;
      if ((m >> (2 * ax + 1) & 1) && x[ax] >= n + 1) return true;
    }
    return false;
  };
  for (int e = 0; e < ne; ++e) {
    const int *G = &GC[4 * (size_t)e + 1], *P = &IP[4 * (size_t)e + 1];
    const int q = case_of(G[0]);
    if (q < 0 || q >= ncs) continue;
    bool hit = case_of(P[0]) != q || in_slab(G[0], G[1], G[2], G[3]);
    for (int dd = 0; dd < 8 && !hit; ++dd)
      hit = in_slab(P[0], P[1] + (dd & 1), P[2] + (dd >> 1 & 1), P[3] + (dd >> 2 & 1));
    if (hit) shared[q] = 1;
  }
}

bool build_push_table(int ncube, const std::vector<FaceTask> &tasks,
                      const std::vector<int> &task_cube, std::vector<int> &push) {
  push.assign(6 * (size_t)std::max(ncube, 0), 0);
  for (size_t t = 0; t < tasks.size(); ++t) {
    const FaceTask &f = tasks[t];
    if (f.kind != 0) continue;
    int &slot = push[6 * (size_t)f.src + 2 * f.axis + (f.side == 1 ? 0 : 1)];
    if (slot != 0 && slot != task_cube[t]) return false;
    slot = task_cube[t];
  }
  return true;
}

}  // namespace bcmg

// ---------------------------------------------------------------------------
// C entry points exposing the table builders (diagnostics and host tests).
// ---------------------------------------------------------------------------
#include "../../include/bcm_gb300.h"

extern "C" int bcmg_ibm_schedule(int nbc, const int *GCindex, const int *IPsur, int n, int ncube,
                                 int *level_of_entry) {
  std::vector<int> order, off;
  std::string err;
  if (nbc < 0 || (nbc > 0 && (!GCindex || !IPsur || !level_of_entry))) return -1;
  if (!bcmg::build_ibm_levels(nbc, GCindex, IPsur, n, ncube, order, off, err)) return -1;
  for (size_t l = 1; l < off.size(); ++l)
    for (int t = off[l - 1]; t < off[l]; ++t) level_of_entry[order[t] - 1] = (int)l;
  return (int)off.size() - 1;
}

extern "C" int bcmg_interface_tasks(int ncube, const int *adj_number, const int *csl,
                                    int *task_off, int *task_words, int max_tasks) {
  std::vector<int> off;
  std::vector<bcmg::FaceTask> tasks;
  std::string err;
  if (ncube < 2 || !adj_number || !csl) return -1;
  if (!bcmg::build_interface_tasks(ncube, adj_number, csl, off, tasks, err)) return -1;
  if ((int)tasks.size() > max_tasks) return -2;
  if (task_off)
    for (size_t i = 0; i < off.size(); ++i) task_off[i] = off[i];
  if (task_words)
    for (size_t t = 0; t < tasks.size(); ++t) {
      task_words[5 * t + 0] = tasks[t].src;
      task_words[5 * t + 1] = tasks[t].axis;
      task_words[5 * t + 2] = tasks[t].side;
      task_words[5 * t + 3] = tasks[t].kind;
      task_words[5 * t + 4] = tasks[t].slot;
    }
  return (int)tasks.size();
}

extern "C" int bcmg_interface_plan(int n, int ncube, const int *adj_number, const int *csl,
                                   const int *const bc_lists[6], const int bc_counts[6],
                                   const int *gc_minus, int nminus, const int *gc_plus, int nplus,
                                   int *keep_prologue, int *push, int max_tasks) {
  std::vector<int> off;
  std::vector<bcmg::FaceTask> tasks;
  std::string err;
  if (ncube < 2 || n < 1 || !adj_number || !csl || !bc_lists || !bc_counts) return -1;
  if (!bcmg::build_interface_tasks(ncube, adj_number, csl, off, tasks, err)) return -1;
  std::vector<int> bcc, bcm;
  if (!bcmg::build_bc_entries(ncube, bc_lists, bc_counts, bcc, bcm, err)) return -1;
  if ((int)tasks.size() > max_tasks) return -2;
  std::vector<int> task_cube(tasks.size());
  for (int c = 1; c < ncube; ++c)
    for (int t = off[c]; t < off[c + 1]; ++t) task_cube[t] = c;
  std::vector<char> keep;
  bcmg::prologue_task_mask(n, ncube, tasks, task_cube, bcc, bcm, gc_minus, nminus, gc_plus, nplus,
                           keep);
  if (keep_prologue)
    for (size_t t = 0; t < keep.size(); ++t) keep_prologue[t] = keep[t];
  std::vector<int> tbl;
  const bool ok = bcmg::build_push_table(ncube, tasks, task_cube, tbl);
  if (push) std::copy(tbl.begin(), tbl.end(), push);
  return ok ? (int)tasks.size() : -3;
}

extern "C" int bcmg_ghost_beside_plan(int n, int ncube, const int *const bc_lists[6],
                                      const int bc_counts[6], const int *gc_minus,
                                      const int *ip_minus, int nminus, const int *gc_plus,
                                      const int *ip_plus, int nplus, const int *case_cube0,
                                      int ncase, int *beside) {
  if (ncube < 2 || n < 1 || !bc_lists || !bc_counts || ncase < 1 || !case_cube0 || !beside)
    return -1;
  std::vector<int> bcc, bcm;
  std::string err;
  if (!bcmg::build_bc_entries(ncube, bc_lists, bc_counts, bcc, bcm, err)) return -1;
  const int ne = std::max(0, nminus) + std::max(0, nplus);
  std::vector<int> gc(4 * (size_t)ne + 1, 0), ip(4 * (size_t)ne + 1, 0);
  if (nminus > 0) {
    if (!gc_minus || !ip_minus) return -1;
    std::copy(gc_minus + 1, gc_minus + 1 + 4 * (size_t)nminus, gc.begin() + 1);
    std::copy(ip_minus + 1, ip_minus + 1 + 4 * (size_t)nminus, ip.begin() + 1);
  }
  if (nplus > 0) {
    if (!gc_plus || !ip_plus) return -1;
    std::copy(gc_plus + 1, gc_plus + 1 + 4 * (size_t)nplus, gc.begin() + 1 + 4 * (size_t)std::max(0, nminus));
    std::copy(ip_plus + 1, ip_plus + 1 + 4 * (size_t)nplus, ip.begin() + 1 + 4 * (size_t)std::max(0, nminus));
  }
  std::vector<int> c0(case_cube0, case_cube0 + ncase + 1);
  std::vector<char> shared;
  bcmg::ghost_shared_cases(n, ncube, bcc, bcm, gc.data(), ip.data(), ne, c0, shared);
  for (int q = 0; q < ncase; ++q) beside[q] = !bcc.empty() && !shared[q];
  return ncase;
}

extern "C" int bcmg_interface_closing_plan(int n, int ncube, const int *adj_number,
                                           const int *csl, const int *const bc_lists[6],
                                           const int bc_counts[6], const int *ip_minus,
                                           int nminus, const int *ip_plus, int nplus,
                                           int *keep_closing, int *edge_cubes, int max_tasks) {
  std::vector<int> off;
  std::vector<bcmg::FaceTask> tasks;
  std::string err;
  if (ncube < 2 || n < 1 || !adj_number || !csl || !bc_lists || !bc_counts) return -1;
  if (!bcmg::build_interface_tasks(ncube, adj_number, csl, off, tasks, err)) return -1;
  std::vector<int> bcc, bcm;
  if (!bcmg::build_bc_entries(ncube, bc_lists, bc_counts, bcc, bcm, err)) return -1;
  if ((int)tasks.size() > max_tasks) return -2;
  std::vector<int> task_cube(tasks.size());
  for (int c = 1; c < ncube; ++c)
    for (int t = off[c]; t < off[c + 1]; ++t) task_cube[t] = c;
  std::vector<char> keep, edge;
  bcmg::closing_plan(n, ncube, tasks, task_cube, bcc, bcm, ip_minus, nminus, ip_plus, nplus, keep,
                     edge);
  if (keep_closing)
    for (size_t t = 0; t < keep.size(); ++t) keep_closing[t] = keep[t];
  if (edge_cubes)
    for (int c = 0; c < ncube; ++c) edge_cubes[c] = edge[c];
  return (int)tasks.size();
}

// ---------------------------------------------------------------------------
// Cube-sharded runs.  The reference spreads cubes over MPI ranks by
// rank_map.dat (main.cpp:576-596) and exchanges the face layers of cubes on
// other ranks every interface call (BCM_Interface.cpp:213-1738,
// :4367-5634).  Here a rank holds its own cubes, then one "proxy" slot per
// remote cube that a face task of one of its cubes reads; before each
// interface call the face bands those tasks read are copied into the proxy
// slots, and the interface kernels run unchanged.
// ---------------------------------------------------------------------------
namespace {

// Face tasks of the global case whose destination is on rank `dst` and whose
// source is on rank `src`, as bands of the source cube: (source cube, axis,
// side of the source's face: 1 = its high face, layers it reads).  A
// same-level copy reads the source's two layers next to the face, an
// injection one (two are sent), a fine -> coarse average four.
bool shard_bands(int ncube, const int *adj, const int *csl, const int *rank_of_cube, int src,
                 int dst, std::vector<std::array<int, 4>> &out, std::string &err) {
  std::vector<int> off;
  std::vector<bcmg::FaceTask> tasks;
  if (!bcmg::build_interface_tasks(ncube, adj, csl, off, tasks, err)) return false;
  std::map<std::array<int, 3>, int> need;  // (cube, axis, side) -> layers
  for (int c = 1; c < ncube; ++c) {
    if (rank_of_cube[c] != dst) continue;
    for (int t = off[c]; t < off[c + 1]; ++t) {
      const bcmg::FaceTask &f = tasks[t];
      if (rank_of_cube[f.src] != src || f.src == c) continue;
      // the task fills the destination's ghost layers on side f.side, so it
      // reads the source's face on the other side
      const std::array<int, 3> key = {f.src, (int)f.axis, 1 - (int)f.side};
      int &l = need[key];
      l = std::max(l, f.kind == 2 ? 4 : 2);
    }
  }
  out.clear();
  for (auto &kv : need) out.push_back({kv.first[0], kv.first[1], kv.first[2], kv.second});
  return true;
}

bool check_ranks(int ncube, const int *rank_of_cube, int rank) {
  if (!rank_of_cube || rank < 0) return false;
  for (int c = 1; c < ncube; ++c)
    if (rank_of_cube[c] < 0) return false;
  return true;
}

}  // namespace

extern "C" int bcmg_shard_plan(int ncube, const int *adj_number, const int *csl,
                               const int *rank_of_cube, int rank, int cap, int *nlocal,
                               int *local_cubes, int *nproxy, int *proxy_cubes) {
  std::string err;
  if (ncube < 2 || !adj_number || !csl || !nlocal || !nproxy ||
      !check_ranks(ncube, rank_of_cube, rank))
    return -1;
  std::vector<int> off;
  std::vector<bcmg::FaceTask> tasks;
  if (!bcmg::build_interface_tasks(ncube, adj_number, csl, off, tasks, err)) return -1;
  std::vector<int> loc, prox;
  std::vector<char> isprox((size_t)ncube, 0);
  for (int c = 1; c < ncube; ++c) {
    if (rank_of_cube[c] != rank) continue;
    loc.push_back(c);
    for (int t = off[c]; t < off[c + 1]; ++t)
      if (rank_of_cube[tasks[t].src] != rank) isprox[tasks[t].src] = 1;
  }
  for (int c = 1; c < ncube; ++c)
    if (isprox[c]) prox.push_back(c);
  *nlocal = (int)loc.size();
  *nproxy = (int)prox.size();
  if ((int)loc.size() > cap || (int)prox.size() > cap) return -2;
  if (local_cubes) std::copy(loc.begin(), loc.end(), local_cubes);
  if (proxy_cubes) std::copy(prox.begin(), prox.end(), proxy_cubes);
  return 0;
}

extern "C" int bcmg_shard_bands(int ncube, const int *adj_number, const int *csl,
                                const int *rank_of_cube, int src_rank, int dst_rank, int cap,
                                int *nband, int *bands) {
  std::string err;
  if (ncube < 2 || !adj_number || !csl || !nband ||
      !check_ranks(ncube, rank_of_cube, std::min(src_rank, dst_rank)))
    return -1;
  std::vector<std::array<int, 4>> b;
  if (!shard_bands(ncube, adj_number, csl, rank_of_cube, src_rank, dst_rank, b, err)) return -1;
  *nband = (int)b.size();
  if ((int)b.size() > cap) return -2;
  if (bands)
    for (size_t i = 0; i < b.size(); ++i)
      for (int w = 0; w < 4; ++w) bands[4 * i + w] = b[i][w];
  return 0;
}
