// The flag field's same-level interface (BCM_FWS_Interface.cpp:23-791) and
// the flag bands of cube-sharded runs, host side.
#pragma once

#include <string>
#include <vector>

namespace bcmg {

// Cubes with a same-level +axis neighbour, per axis, classified like
// BCM_Interface_table.cpp:96-120 (a relation when any of the four slots
// adj_number[c][1..4][dir] is positive; the classifying cube is the largest
// slot value; same level when csl matches).
bool same_level_pairs(int ncube, const int *adj, const int *csl, std::vector<int> pairs[3],
                      std::string &err);

// BCM_FWS_Interface on one rank for the given pair lists (the +axis
// neighbour of pairs[ax][*] is slot 1 of adj_number, as the reference reads
// it): same-level ghost-face copies, sign threshold and hole fill of every
// finest-level cube, in place on FWS[ncube][n+4]^3.
bool fws_interface(int n, int ncube, const int *csl, const int *adj,
                   const std::vector<int> pairs[3], int *FWS, std::string &err);

// Packs (unpack = false) or unpacks flag bands in the band convention of the
// state halo: 4 ints per band (cube slot, axis, side 1 high / 0 low, layers),
// the band's cells in (layer, first in-face index, second) order.
bool fws_bands(int n, int ncube, int *FWS, int nband, const int *bands, int *buf, bool unpack,
               std::string &err);

}  // namespace bcmg
