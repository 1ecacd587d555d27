// Tecplot ASCII output of the corner fields, in the format of the reference's
// mesh writer (outputMeshDataTECPLOT, src/meshAMR/meshAMRgeneric.h:8845, data
// file layout :7685-7710): a VARIABLES line, one ZONE with
// DATAPACKING=POINT, ZONETYPE=FEBRICK of N nodes and E cells, one line per
// node (its position, then its values, each "%e"), then per cell the 8 node
// numbers (1-based) in the brick order (0,0,0) (1,0,0) (1,1,0) (0,1,0)
// (0,0,1) (1,0,1) (1,1,1) (0,1,1).  The values are ECSIM's corner-node
// output -- E ("Ex (corner node)", pic_field_solver_ecsim.cpp:6416-6420) --
// followed by the corner B and E^{n+theta}.
//
// Nodes are the corners of the cells at their positions: on a periodic mesh
// the far faces get their own nodes carrying the values of the corners they
// wrap to, so every brick is local; on an AMR mesh the nodes are the distinct
// corner positions of the leaf blocks (hanging corners included), the values
// those of the unique corner the block's corner table names.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.cuh"

namespace {

// brick corner order of the writer
constexpr int kBrick[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                              {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

}  // namespace

extern "C" amps_gpu_status amps_gpu_write_tecplot(amps_gpu_ctx* c, const char* path) {
  if (!c || !path) return set_err(c, AMPS_GPU_INVALID_ARG, "write_tecplot: null argument");
  const long long nv = c->nvc, ncell = c->ncor;
  std::vector<double> En(3 * nv), Eh(3 * nv), Bp(3 * nv), Bc(3 * nv), Bcen(3 * ncell);
  amps_gpu_status st = amps_gpu_export_fields(c, En.data(), Eh.data(), Bcen.data(), Bp.data(), Bc.data());
  if (st) return st;
  // node positions (finest-lattice or cell-lattice integers), the unique corner
  // each node takes its values from, and the 8 nodes of every cell
  std::vector<long long> pos;   // 3 per node
  std::vector<long long> src;   // unique corner per node
  std::vector<long long> conn((size_t)ncell * 8);
  double x0[3], h[3];
  if (!c->amr) {
    const int N[3] = {8 * c->cfg.nbx, 8 * c->cfg.nby, 8 * c->cfg.nbz};
    for (int d = 0; d < 3; d++) { x0[d] = c->cfg.x0[d]; h[d] = c->cfg.dx[d]; }
    const long long N1[3] = {N[0] + 1LL, N[1] + 1LL, N[2] + 1LL};
    for (long long K = 0; K < N1[2]; K++)
      for (long long J = 0; J < N1[1]; J++)
        for (long long I = 0; I < N1[0]; I++) {
          pos.push_back(I); pos.push_back(J); pos.push_back(K);
          src.push_back((I % N[0]) + (long long)N[0] * ((J % N[1]) + (long long)N[1] * (K % N[2])));
        }
    for (int b = 0; b < c->nb; b++) {
      const int bx = b % c->cfg.nbx, by = (b / c->cfg.nbx) % c->cfg.nby, bz = b / (c->cfg.nbx * c->cfg.nby);
      for (int l = 0; l < AMPS_CPB; l++) {
        const long long I = 8 * bx + (l & 7), J = 8 * by + ((l >> 3) & 7), K = 8 * bz + (l >> 6);
        for (int q = 0; q < 8; q++)
          conn[((size_t)b * AMPS_CPB + l) * 8 + q] =
              (I + kBrick[q][0]) + N1[0] * ((J + kBrick[q][1]) + N1[1] * (K + kBrick[q][2]));
      }
    }
  } else {
    std::vector<int> ctab((size_t)c->nb * 729), borg((size_t)c->nb * 3), bscale(c->nb);
    cudaError_t e = cudaMemcpy(ctab.data(), c->d_ctab, sizeof(int) * ctab.size(), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(borg.data(), c->d_borg, sizeof(int) * borg.size(), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(bscale.data(), c->d_bscale, sizeof(int) * bscale.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_check(c, e, "write_tecplot: mesh tables");
    for (int d = 0; d < 3; d++) { x0[d] = c->cfg.x0[d]; h[d] = c->dxf; }
    std::unordered_map<long long, long long> id;   // finest-lattice position -> node
    const long long M = 1LL << 21;                 // key stride (lattice sizes are far below)
    for (int b = 0; b < c->nb; b++)
      for (int l = 0; l < AMPS_CPB; l++) {
        const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
        for (int q = 0; q < 8; q++) {
          const int ci = i + kBrick[q][0], cj = j + kBrick[q][1], ck = k + kBrick[q][2];
          const long long g[3] = {borg[3 * b] + (long long)ci * bscale[b],
                                  borg[3 * b + 1] + (long long)cj * bscale[b],
                                  borg[3 * b + 2] + (long long)ck * bscale[b]};
          const long long key = g[0] + M * (g[1] + M * g[2]);
          auto it = id.find(key);
          long long node;
          if (it == id.end()) {
            node = (long long)src.size();
            id.emplace(key, node);
            pos.push_back(g[0]); pos.push_back(g[1]); pos.push_back(g[2]);
            src.push_back(ctab[(size_t)b * 729 + ci + 9 * (cj + 9 * ck)]);
          } else {
            node = it->second;
          }
          conn[((size_t)b * AMPS_CPB + l) * 8 + q] = node;
        }
      }
  }
  FILE* f = fopen(path, "w");
  if (!f) return set_err(c, AMPS_GPU_INVALID_ARG, std::string("write_tecplot: cannot open ") + path);
  const long long nn = (long long)src.size();
  fprintf(f, "VARIABLES=\"X\", \"Y\", \"Z\"");
  fprintf(f, ",\"Ex (corner node)\",\"Ey (corner node)\",\"Ez (corner node)\"");
  fprintf(f, ",\"Bx (corner node)\",\"By (corner node)\",\"Bz (corner node)\"");
  fprintf(f, ",\"Ex theta (corner node)\",\"Ey theta (corner node)\",\"Ez theta (corner node)\"");
  fprintf(f, "\nZONE N=%lld, E=%lld, DATAPACKING=POINT, ZONETYPE=FEBRICK\n", nn, ncell);
  // the export layout is interleaved x, y, z per corner
  for (long long n = 0; n < nn; n++) {
    const long long s = src[(size_t)n];
    fprintf(f, "%e  %e  %e  ", x0[0] + pos[3 * n] * h[0], x0[1] + pos[3 * n + 1] * h[1],
            x0[2] + pos[3 * n + 2] * h[2]);
    fprintf(f, "%e %e %e ", En[3 * s], En[3 * s + 1], En[3 * s + 2]);
    fprintf(f, "%e %e %e ", Bc[3 * s], Bc[3 * s + 1], Bc[3 * s + 2]);
    fprintf(f, "%e %e %e\n", Eh[3 * s], Eh[3 * s + 1], Eh[3 * s + 2]);
  }
  for (long long e = 0; e < ncell; e++) {
    const long long* q = &conn[(size_t)e * 8];
    fprintf(f, "%lld %lld %lld %lld %lld %lld %lld %lld\n", q[0] + 1, q[1] + 1, q[2] + 1, q[3] + 1,
            q[4] + 1, q[5] + 1, q[6] + 1, q[7] + 1);
  }
  const bool ok = ferror(f) == 0;
  fclose(f);
  return ok ? AMPS_GPU_OK : set_err(c, AMPS_GPU_INVALID_ARG, "write_tecplot: write failed");
}
