// Host-side builder of 2:1-balanced, periodic, block-structured AMR meshes
// (the leaf blocks of the reference's octree, src/meshAMR/meshAMRgeneric.h).
//
// Input: leaf blocks of 8^3 cells, each with a refinement level and its origin
// on the finest lattice (finest-cell units).  Output tables:
//   * block geometry (origin, cell size), and a finest-block -> leaf map that
//     replaces findTreeNode's tree walk (meshAMRgeneric.h:2793-2885);
//   * unique corners (corners shared by blocks are one entry) with, per block,
//     a 9^3 table block-local corner -> unique corner;
//   * hanging corners: corners of a fine block that lie on the face or edge of
//     a coarser neighbour without being one of its corners.  Their values are
//     constrained to the multilinear interpolation of the coarser block's
//     corners (weights 1/2 or 1/4, expanded recursively until every parent is
//     a free corner).
// The reference's ECSIM assumes same-level neighbours (GetStencil,
// src/pic/ecsim/get_stencil.cpp:1100-1160); these constraints are what makes
// the cell-assembled operator conforming across resolution jumps.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "amr_mesh.h"

namespace {

inline int wrapi(int v, int n) {
  v %= n;
  return v < 0 ? v + n : v;
}

inline uint64_t key3(int x, int y, int z) {
  return ((uint64_t)(uint32_t)x << 42) | ((uint64_t)(uint32_t)y << 21) | (uint64_t)(uint32_t)z;
}

}  // namespace

extern "C" amps_gpu_status amps_amr_build(int nbx0, int nby0, int nbz0, int lmax,
                                          const double* x0, double dx0,
                                          const amps_block_desc* blocks, int nblocks,
                                          amps_amr_mesh** out) {
  return amps_amr_build_open(nbx0, nby0, nbz0, lmax, x0, dx0, blocks, nblocks, nullptr, 0, out);
}

extern "C" amps_gpu_status amps_amr_build_open(int nbx0, int nby0, int nbz0, int lmax,
                                               const double* x0, double dx0,
                                               const amps_block_desc* blocks, int nblocks,
                                               const int* open_axes, int field_bc,
                                               amps_amr_mesh** out) {
  const int faces[6] = {field_bc, field_bc, field_bc, field_bc, field_bc, field_bc};
  return amps_amr_build_open_faces(nbx0, nby0, nbz0, lmax, x0, dx0, blocks, nblocks, open_axes,
                                   faces, out);
}

extern "C" amps_gpu_status amps_amr_build_open_faces(int nbx0, int nby0, int nbz0, int lmax,
                                                     const double* x0, double dx0,
                                                     const amps_block_desc* blocks, int nblocks,
                                                     const int* open_axes, const int* face_bc,
                                                     amps_amr_mesh** out) {
  if (!out || !blocks || nblocks <= 0 || nbx0 <= 0 || nby0 <= 0 || nbz0 <= 0 || lmax < 0 ||
      lmax > 6 || dx0 <= 0.0 || !face_bc)
    return AMPS_GPU_INVALID_ARG;
  for (int f = 0; f < 6; f++)
    if (face_bc[f] < 0 || face_bc[f] > 1) return AMPS_GPU_INVALID_ARG;
  *out = nullptr;
  amps_amr_mesh* m = new amps_amr_mesh();
  for (int d = 0; d < 3; d++) m->open[d] = open_axes && open_axes[d] ? 1 : 0;
  // the Neumann faces of the open axes (cDomainBC's per-face policy,
  // src/pic/ecsim/domain_bc.cpp:39-45)
  for (int f = 0; f < 6; f++)
    if (m->open[f / 2] && face_bc[f] == 1) m->neumann |= 1 << f;
  // periodic axes wrap lattice positions; open axes keep them (corners 0..nfine)
  auto wrap = [&](int d, int v) { return m->open[d] ? v : wrapi(v, m->nfine[d]); };
  m->nb0[0] = nbx0; m->nb0[1] = nby0; m->nb0[2] = nbz0;
  m->lmax = lmax;
  for (int d = 0; d < 3; d++) m->x0[d] = x0 ? x0[d] : 0.0;
  m->dx0 = dx0;
  const int r = 1 << lmax;
  for (int d = 0; d < 3; d++) m->nfine[d] = m->nb0[d] * 8 * r;
  const int nfb[3] = {m->nb0[0] * r, m->nb0[1] * r, m->nb0[2] * r};  // finest blocks per axis
  m->blocks.assign(blocks, blocks + nblocks);
  // coverage map
  m->fine_map.assign((size_t)nfb[0] * nfb[1] * nfb[2], -1);
  for (int b = 0; b < nblocks; b++) {
    const amps_block_desc& B = blocks[b];
    if (B.level < 0 || B.level > lmax) { delete m; return AMPS_GPU_INVALID_ARG; }
    const int size = 8 << (lmax - B.level);  // finest cells per edge
    const int o[3] = {B.ix, B.iy, B.iz};
    for (int d = 0; d < 3; d++)
      if (o[d] < 0 || o[d] % size != 0 || o[d] + size > m->nfine[d]) { delete m; return AMPS_GPU_INVALID_ARG; }
    const int nfbb = size / 8;
    for (int k = 0; k < nfbb; k++)
      for (int j = 0; j < nfbb; j++)
        for (int i = 0; i < nfbb; i++) {
          const size_t idx = (size_t)(o[0] / 8 + i) + (size_t)nfb[0] * ((o[1] / 8 + j) + (size_t)nfb[1] * (o[2] / 8 + k));
          if (m->fine_map[idx] != -1) { delete m; return AMPS_GPU_INVALID_ARG; }  // overlap
          m->fine_map[idx] = b;
        }
  }
  for (int32_t v : m->fine_map)
    if (v < 0) { delete m; return AMPS_GPU_INVALID_ARG; }  // gap
  auto block_at = [&](int X, int Y, int Z) {  // leaf block covering finest cell (X,Y,Z), -1 outside
    X = wrap(0, X); Y = wrap(1, Y); Z = wrap(2, Z);
    if (X < 0 || X >= m->nfine[0] || Y < 0 || Y >= m->nfine[1] || Z < 0 || Z >= m->nfine[2]) return -1;
    return (int)m->fine_map[(size_t)(X / 8) + (size_t)nfb[0] * ((Y / 8) + (size_t)nfb[1] * (Z / 8))];
  };
  // 2:1 balance across faces, edges and vertices
  for (int b = 0; b < nblocks; b++) {
    const amps_block_desc& B = blocks[b];
    const int size = 8 << (lmax - B.level);
    for (int oz = -1; oz <= 1; oz++)
      for (int oy = -1; oy <= 1; oy++)
        for (int ox = -1; ox <= 1; ox++) {
          const int X = B.ix + (ox < 0 ? -1 : (ox > 0 ? size : 0));
          const int Y = B.iy + (oy < 0 ? -1 : (oy > 0 ? size : 0));
          const int Z = B.iz + (oz < 0 ? -1 : (oz > 0 ? size : 0));
          const int nbk = block_at(X, Y, Z);
          if (nbk >= 0 && std::abs(blocks[nbk].level - B.level) > 1) { delete m; return AMPS_GPU_INVALID_ARG; }
        }
  }
  // unique corners
  std::unordered_map<uint64_t, int32_t> id;
  id.reserve((size_t)nblocks * 729);
  m->corner_tab.resize((size_t)nblocks * 729);
  for (int b = 0; b < nblocks; b++) {
    const amps_block_desc& B = blocks[b];
    const int st = 1 << (lmax - B.level);
    for (int k = 0; k <= 8; k++)
      for (int j = 0; j <= 8; j++)
        for (int i = 0; i <= 8; i++) {
          const int X = wrap(0, B.ix + i * st);
          const int Y = wrap(1, B.iy + j * st);
          const int Z = wrap(2, B.iz + k * st);
          const uint64_t kk = key3(X, Y, Z);
          auto it = id.find(kk);
          int32_t c;
          if (it == id.end()) {
            c = (int32_t)(m->corner_xyz.size() / 3);
            id.emplace(kk, c);
            m->corner_xyz.push_back(X);
            m->corner_xyz.push_back(Y);
            m->corner_xyz.push_back(Z);
          } else {
            c = it->second;
          }
          m->corner_tab[(size_t)b * 729 + i + 9 * (j + 9 * k)] = c;
        }
  }
  const int nc = (int)(m->corner_xyz.size() / 3);
  // hanging corners: a corner is hanging when a coarser leaf block touching it
  // has it off its own corner lattice
  std::vector<std::vector<std::pair<int32_t, double>>> par((size_t)nc);
  std::vector<char> hanging((size_t)nc, 0);
  for (int c = 0; c < nc; c++) {
    const int X = m->corner_xyz[3 * c], Y = m->corner_xyz[3 * c + 1], Z = m->corner_xyz[3 * c + 2];
    int best = -1, best_level = 99;
    // the (up to) 8 finest cells around the corner identify the touching blocks
    for (int dz = -1; dz <= 0; dz++)
      for (int dy = -1; dy <= 0; dy++)
        for (int dx = -1; dx <= 0; dx++) {
          const int b = block_at(X + dx, Y + dy, Z + dz);
          if (b >= 0 && blocks[b].level < best_level) { best_level = blocks[b].level; best = b; }
        }
    const amps_block_desc& B = blocks[best];
    const int st = 1 << (lmax - B.level);
    // position relative to the coarsest touching block (periodic axes wrap)
    const int rel[3] = {m->open[0] ? X - B.ix : wrapi(X - B.ix, m->nfine[0]),
                        m->open[1] ? Y - B.iy : wrapi(Y - B.iy, m->nfine[1]),
                        m->open[2] ? Z - B.iz : wrapi(Z - B.iz, m->nfine[2])};
    bool off = false;
    for (int d = 0; d < 3; d++) off |= (rel[d] % st) != 0;
    if (!off) continue;
    hanging[c] = 1;
    // parents: lattice points of block `best` around the corner
    int lo[3], hi[3];
    for (int d = 0; d < 3; d++) {
      const int q = rel[d] / st, rm = rel[d] - q * st;
      lo[d] = q;
      hi[d] = rm ? q + 1 : q;
    }
    std::vector<std::pair<int32_t, double>> pl;
    int nd = 0;
    for (int d = 0; d < 3; d++) nd += (lo[d] != hi[d]);
    const double w = 1.0 / (1 << nd);
    for (int kz = lo[2]; kz <= hi[2]; kz++)
      for (int jy = lo[1]; jy <= hi[1]; jy++)
        for (int ix = lo[0]; ix <= hi[0]; ix++) {
          if (ix < 0 || ix > 8 || jy < 0 || jy > 8 || kz < 0 || kz > 8) { delete m; return AMPS_GPU_INVALID_ARG; }
          pl.push_back({m->corner_tab[(size_t)best * 729 + ix + 9 * (jy + 9 * kz)], w});
        }
    par[(size_t)c] = pl;
  }
  // expand chains (a parent that is itself hanging) until all parents are free
  for (int c = 0; c < nc; c++) {
    if (!hanging[c]) continue;
    for (int pass = 0; pass < 8; pass++) {
      bool changed = false;
      std::map<int32_t, double> acc;
      for (auto& pw : par[(size_t)c]) {
        if (hanging[pw.first]) {
          for (auto& q : par[(size_t)pw.first]) acc[q.first] += pw.second * q.second;
          changed = true;
        } else {
          acc[pw.first] += pw.second;
        }
      }
      par[(size_t)c].assign(acc.begin(), acc.end());
      if (!changed) break;
    }
  }
  m->hang_start.assign((size_t)nc + 1, 0);
  for (int c = 0; c < nc; c++) {
    m->hang_start[(size_t)c + 1] = m->hang_start[(size_t)c] + (hanging[c] ? (int)par[(size_t)c].size() : 0);
    if (hanging[c])
      for (auto& pw : par[(size_t)c]) {
        m->hang_parent.push_back(pw.first);
        m->hang_weight.push_back(pw.second);
      }
  }
  // boundary rows: free corners on a domain face of an open axis
  // (CollectAndMarkDomainBoundary*CornerNodesOnFaces, GetStencil's
  // boundary_short_circuit, src/pic/ecsim/get_stencil.cpp:440-620): Dirichlet
  // dE_b = 0; Neumann dE_b = mean of one donor per touching face, the corner
  // one step of the finest touching block inward along that face's normal.  A
  // corner on faces of both types is Neumann: RecomputeBCType marks the
  // Dirichlet faces first and the Neumann faces over them
  // (src/pic/ecsim/domain_bc.cpp:49-63).
  m->bnd_flag.assign((size_t)nc, 0);
  m->bnd_start.assign((size_t)nc + 1, 0);
  for (int c = 0; c < nc; c++) {
    m->bnd_start[(size_t)c + 1] = m->bnd_start[(size_t)c];
    if (hanging[c]) continue;
    const int P[3] = {m->corner_xyz[3 * c], m->corner_xyz[3 * c + 1], m->corner_xyz[3 * c + 2]};
    int side[3] = {0, 0, 0}, nface = 0;
    for (int d = 0; d < 3; d++) {
      if (!m->open[d]) continue;
      if (P[d] == 0) side[d] = -1;
      else if (P[d] == m->nfine[d]) side[d] = 1;
      nface += side[d] != 0;
    }
    if (!nface) continue;
    m->bnd_flag[(size_t)c] = 1;
    bool neumann = false;
    for (int d = 0; d < 3; d++)
      if (side[d]) neumann |= (m->neumann >> (2 * d + (side[d] > 0))) & 1;
    if (!neumann) continue;
    int stf = 1 << 30;  // lattice step of the finest block touching the corner
    for (int dz = -1; dz <= 0; dz++)
      for (int dy = -1; dy <= 0; dy++)
        for (int dx = -1; dx <= 0; dx++) {
          const int b = block_at(P[0] + dx, P[1] + dy, P[2] + dz);
          if (b >= 0) stf = std::min(stf, 1 << (lmax - blocks[b].level));
        }
    std::map<int32_t, double> acc;
    for (int d = 0; d < 3; d++) {
      if (!side[d]) continue;
      int Q[3] = {P[0], P[1], P[2]};
      Q[d] -= side[d] * stf;
      auto it = id.find(key3(wrap(0, Q[0]), wrap(1, Q[1]), wrap(2, Q[2])));
      if (it == id.end()) { delete m; return AMPS_GPU_INVALID_ARG; }
      const int32_t q = it->second;
      const double w = 1.0 / nface;
      if (hanging[q]) {
        for (auto& pw : par[(size_t)q]) acc[pw.first] += w * pw.second;
      } else {
        acc[q] += w;
      }
    }
    for (auto& cw : acc) {
      m->bnd_col.push_back(cw.first);
      m->bnd_weight.push_back(cw.second);
    }
    m->bnd_start[(size_t)c + 1] = (int32_t)m->bnd_col.size();
  }
  *out = m;
  return AMPS_GPU_OK;
}

extern "C" amps_gpu_status amps_amr_boundary_tables(const amps_amr_mesh* m, int* nentries, int32_t* flag,
                                                    int32_t* start, int32_t* col, double* weight) {
  if (!m) return AMPS_GPU_INVALID_ARG;
  if (nentries) *nentries = (int)m->bnd_col.size();
  auto cp = [](auto* dst, const auto& v) {
    if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
  };
  cp(flag, m->bnd_flag);
  cp(start, m->bnd_start);
  cp(col, m->bnd_col);
  cp(weight, m->bnd_weight);
  return AMPS_GPU_OK;
}

extern "C" amps_gpu_status amps_amr_info(const amps_amr_mesh* m, int* nblocks, int* ncorners,
                                         int* nhanging, int* nparents, int* nfine) {
  if (!m) return AMPS_GPU_INVALID_ARG;
  if (nblocks) *nblocks = (int)m->blocks.size();
  const int nc = (int)(m->corner_xyz.size() / 3);
  if (ncorners) *ncorners = nc;
  if (nhanging) {
    int h = 0;
    for (int c = 0; c < nc; c++) h += m->hang_start[(size_t)c + 1] > m->hang_start[(size_t)c];
    *nhanging = h;
  }
  if (nparents) *nparents = (int)m->hang_parent.size();
  if (nfine)
    for (int d = 0; d < 3; d++) nfine[d] = m->nfine[d];
  return AMPS_GPU_OK;
}

// Copies the tables out (any pointer may be NULL): corner_tab[nblocks*729],
// corner_xyz[3*ncorners], hang_start[ncorners+1], hang_parent[nparents],
// hang_weight[nparents], fine_map[finest blocks].
extern "C" amps_gpu_status amps_amr_tables(const amps_amr_mesh* m, int32_t* corner_tab,
                                           int32_t* corner_xyz, int32_t* hang_start,
                                           int32_t* hang_parent, double* hang_weight,
                                           int32_t* fine_map) {
  if (!m) return AMPS_GPU_INVALID_ARG;
  auto cp = [](auto* dst, const auto& v) {
    if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0]));
  };
  cp(corner_tab, m->corner_tab);
  cp(corner_xyz, m->corner_xyz);
  cp(hang_start, m->hang_start);
  cp(hang_parent, m->hang_parent);
  cp(hang_weight, m->hang_weight);
  cp(fine_map, m->fine_map);
  return AMPS_GPU_OK;
}

extern "C" amps_gpu_status amps_amr_destroy(amps_amr_mesh* m) {
  delete m;
  return AMPS_GPU_OK;
}

// Leaf blocks of the nested-refinement meshes used by the AMR workloads:
// mode 0: blocks whose centre lies in the central box |x - c| < frac*L/2 on
//         every axis are refined, level by level (the box half-width shrinks
//         by half per level);
// mode 1: blocks that intersect the sphere |x - c| < radius_frac*L are refined
//         (radius halves per level); 2:1 balance is enforced by refining the
//         neighbours of too-fine blocks.
// Returns the number of leaves (or a negative status); fills up to cap.
extern "C" int amps_amr_nested_leaves(int nbx0, int nby0, int nbz0, int lmax, int mode,
                                      double frac, amps_block_desc* out, int cap) {
  if (nbx0 <= 0 || nby0 <= 0 || nbz0 <= 0 || lmax < 0 || lmax > 6) return -AMPS_GPU_INVALID_ARG;
  const int nfine[3] = {nbx0 * 8 << lmax, nby0 * 8 << lmax, nbz0 * 8 << lmax};
  struct Leaf { int level, ix, iy, iz; };
  std::vector<Leaf> cur;
  for (int k = 0; k < nbz0; k++)
    for (int j = 0; j < nby0; j++)
      for (int i = 0; i < nbx0; i++) cur.push_back({0, i * (8 << lmax), j * (8 << lmax), k * (8 << lmax)});
  auto wants = [&](const Leaf& B, int level_next) {
    const int size = 8 << (lmax - B.level);
    double mn = 1e300;
    double lo[3] = {(double)B.ix, (double)B.iy, (double)B.iz};
    double hi[3] = {lo[0] + size, lo[1] + size, lo[2] + size};
    if (mode == 0) {
      const double hw = frac / (1 << (level_next - 1)) * 0.5;
      bool in = true;
      for (int d = 0; d < 3; d++) {
        const double c = (lo[d] + hi[d]) * 0.5 / nfine[d];
        in = in && std::abs(c - 0.5) < hw;
      }
      return in;
    }
    // sphere: distance from the domain centre to the block box (relative units)
    double d2 = 0.0;
    for (int d = 0; d < 3; d++) {
      const double c = 0.5 * nfine[d];
      const double q = std::max(lo[d] - c, std::max(0.0, c - hi[d])) / nfine[d];
      d2 += q * q;
    }
    mn = std::sqrt(d2);
    return mn < frac / (1 << (level_next - 1));
  };
  for (int lev = 1; lev <= lmax; lev++) {
    std::vector<Leaf> nxt;
    for (auto& B : cur) {
      if (B.level == lev - 1 && wants(B, lev)) {
        const int h = 4 << (lmax - B.level);
        for (int c = 0; c < 8; c++)
          nxt.push_back({lev, B.ix + (c & 1) * h, B.iy + ((c >> 1) & 1) * h, B.iz + ((c >> 2) & 1) * h});
      } else {
        nxt.push_back(B);
      }
    }
    cur.swap(nxt);
  }
  // enforce 2:1 balance by refining coarse neighbours of fine blocks
  for (int pass = 0; pass < 16; pass++) {
    const int nfb[3] = {nfine[0] / 8, nfine[1] / 8, nfine[2] / 8};
    std::vector<int> map((size_t)nfb[0] * nfb[1] * nfb[2], -1);
    for (size_t b = 0; b < cur.size(); b++) {
      const int nfbb = 1 << (lmax - cur[b].level);
      for (int k = 0; k < nfbb; k++)
        for (int j = 0; j < nfbb; j++)
          for (int i = 0; i < nfbb; i++)
            map[(size_t)(cur[b].ix / 8 + i) + (size_t)nfb[0] * ((cur[b].iy / 8 + j) + (size_t)nfb[1] * (cur[b].iz / 8 + k))] = (int)b;
    }
    std::vector<char> refine(cur.size(), 0);
    for (size_t b = 0; b < cur.size(); b++) {
      const int size = 8 << (lmax - cur[b].level);
      for (int oz = -1; oz <= 1; oz++)
        for (int oy = -1; oy <= 1; oy++)
          for (int ox = -1; ox <= 1; ox++) {
            int X = cur[b].ix + (ox < 0 ? -1 : (ox > 0 ? size : 0));
            int Y = cur[b].iy + (oy < 0 ? -1 : (oy > 0 ? size : 0));
            int Z = cur[b].iz + (oz < 0 ? -1 : (oz > 0 ? size : 0));
            X = (X % nfine[0] + nfine[0]) % nfine[0];
            Y = (Y % nfine[1] + nfine[1]) % nfine[1];
            Z = (Z % nfine[2] + nfine[2]) % nfine[2];
            const int nb = map[(size_t)(X / 8) + (size_t)nfb[0] * ((Y / 8) + (size_t)nfb[1] * (Z / 8))];
            if (cur[nb].level < cur[b].level - 1) refine[nb] = 1;
          }
    }
    bool any = false;
    std::vector<Leaf> nxt;
    for (size_t b = 0; b < cur.size(); b++) {
      if (refine[b]) {
        any = true;
        const int h = 4 << (lmax - cur[b].level);
        for (int c = 0; c < 8; c++)
          nxt.push_back({cur[b].level + 1, cur[b].ix + (c & 1) * h, cur[b].iy + ((c >> 1) & 1) * h,
                         cur[b].iz + ((c >> 2) & 1) * h});
      } else {
        nxt.push_back(cur[b]);
      }
    }
    cur.swap(nxt);
    if (!any) break;
  }
  const int n = (int)cur.size();
  if (out)
    for (int b = 0; b < n && b < cap; b++) out[b] = {cur[b].level, cur[b].ix, cur[b].iy, cur[b].iz};
  return n;
}
