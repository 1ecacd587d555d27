// Host representation of a block-structured AMR mesh (built by amr.cpp, read by
// the context creator in capi.cu).
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/amps_gpu.h"

struct amps_amr_mesh {
  int nb0[3] = {0, 0, 0};      // level-0 blocks per axis
  int lmax = 0;
  double x0[3] = {0, 0, 0};
  double dx0 = 1.0;            // level-0 cell size
  int nfine[3] = {0, 0, 0};    // finest cells per axis
  std::vector<amps_block_desc> blocks;
  std::vector<int32_t> fine_map;       // finest-block index -> leaf block
  std::vector<int32_t> corner_tab;     // nblocks * 729
  std::vector<int32_t> corner_xyz;     // ncorners * 3 (finest lattice)
  std::vector<int32_t> hang_start;     // ncorners + 1 (CSR of parents; empty range = free)
  std::vector<int32_t> hang_parent;
  std::vector<double> hang_weight;
  std::string err;
};
