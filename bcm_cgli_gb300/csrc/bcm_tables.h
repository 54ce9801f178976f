// Host-side launch-table builders (see bcm_tables.cpp).
#pragma once

#include <string>
#include <vector>

#include "bcm_kernels.h"

namespace bcmg {

bool build_interface_tasks(int ncube, const int *adj, const int *csl, std::vector<int> &off,
                           std::vector<FaceTask> &tasks, std::string &err);
// lists[3*ax + {0,1,2}] = same-level, big->small (+ax), big->small (-ax)
// lists of axis ax (1-based arrays, counts[]) as BCM_Interface receives them.
bool build_interface_tasks_from_lists(int ncube, const int *adj, const int *csl,
                                      const int *const lists[9], const int counts[9],
                                      std::vector<int> &off, std::vector<FaceTask> &tasks,
                                      std::string &err);
bool build_bc_entries(int ncube, const int *const lists[6], const int counts[6],
                      std::vector<int> &cubes, std::vector<int> &masks, std::string &err);
bool build_ibm_levels(int nbc, const int *GC, const int *IP, int n, int ncube,
                      std::vector<int> &order, std::vector<int> &level_off, std::string &err);
// Which face tasks the interface call ahead of a stage must repeat right
// after the previous stage's closing call: keep[t] = 1 for level-jump tasks,
// for faces the boundary fill writes (bc cubes/masks as build_bc_entries
// makes them) and for faces whose destination ghost layers or source
// interior layers hold an IBM ghost cell (GC tables 1-based, 4 ints per
// entry: cube, i, j, k).
void prologue_task_mask(int n, int ncube, const std::vector<FaceTask> &tasks,
                        const std::vector<int> &task_cube, const std::vector<int> &bc_cubes,
                        const std::vector<int> &bc_masks, const int *gc_minus, int nminus,
                        const int *gc_plus, int nplus, std::vector<char> &keep);
// The closing interface call of split RK stages 1 and 2: keep[t] for the
// level-jump tasks whose ghost face the next stage's boundary fill or an
// IBM stencil (IP tables 1-based) reads before the next opening call
// rewrites it; edge[c] for the cubes whose edge cells such a read sees.
void closing_plan(int n, int ncube, const std::vector<FaceTask> &tasks,
                  const std::vector<int> &task_cube, const std::vector<int> &bc_cubes,
                  const std::vector<int> &bc_masks, const int *ip_minus, int nminus,
                  const int *ip_plus, int nplus, std::vector<char> &keep,
                  std::vector<char> &edge);
// Per case: whether its IBM ghost fill must follow the boundary fill (an
// entry's ghost or stencil cell lies in the layers the boundary fill
// touches, or its stencil is in another case).  GC/IP 1-based, ne entries,
// case_cube0: first cube of each case plus one past the last.
void ghost_shared_cases(int n, int ncube, const std::vector<int> &bc_cubes,
                        const std::vector<int> &bc_masks, const int *GC, const int *IP, int ne,
                        const std::vector<int> &case_cube0, std::vector<char> &shared);
// Same-level push table of the split flux kernel (FluxSplitArgs::push):
// push[6 src + 2 axis + 0] = destination of the task copying src's layers
// 2, 3 (its side 1), push[6 src + 2 axis + 1] = destination of the task
// copying layers n, n+1 (side 0).  False when one slot would need two
// destinations.
bool build_push_table(int ncube, const std::vector<FaceTask> &tasks,
                      const std::vector<int> &task_cube, std::vector<int> &push);

}  // namespace bcmg
