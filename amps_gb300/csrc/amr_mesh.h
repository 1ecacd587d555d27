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
  // non-periodic (open) axes: the corners on their domain faces carry the field
  // boundary condition as constraint rows b: x_b - sum_k w_k x_col_k = 0
  // (Dirichlet: no entries; Neumann: the inward face-normal donors, averaged,
  // hanging donors expanded to their parents)
  int open[3] = {0, 0, 0};
  int neumann = 0;                     // bit 2d + high: Neumann face of open axis d (else Dirichlet)
  std::vector<int32_t> bnd_flag;       // ncorners: 1 on a constraint row
  std::vector<int32_t> bnd_start;      // ncorners + 1
  std::vector<int32_t> bnd_col;
  std::vector<double> bnd_weight;
  std::string err;
};
