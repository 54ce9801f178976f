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

}  // namespace bcmg
