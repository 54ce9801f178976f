// Host-side launch-table builders (see bcm_tables.cpp).
#pragma once

#include <string>
#include <vector>

#include "bcm_kernels.h"

namespace bcmg {

bool build_interface_tasks(int ncube, const int *adj, const int *csl, std::vector<int> &off,
                           std::vector<FaceTask> &tasks, std::string &err);
bool build_interface_tasks_from_lists(int ncube, const int *adj, const int *const lists[3],
                                      const int counts[3], std::vector<int> &off,
                                      std::vector<FaceTask> &tasks, std::string &err);
bool build_bc_entries(int ncube, const int *const lists[6], const int counts[6],
                      std::vector<int> &cubes, std::vector<int> &masks, std::string &err);
bool build_ibm_levels(int nbc, const int *GC, const int *IP, int n, int ncube,
                      std::vector<int> &order, std::vector<int> &level_off, std::string &err);

}  // namespace bcmg
