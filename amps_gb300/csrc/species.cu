// Species moments on corners: the _PIC_FIELD_SOLVER_SAMPLE_SPECIES_ON_CORNER_
// sampling of ProcessCell (src/pic/pic_field_solver_ecsim.cpp:2270-2303, flush
// :2384-2394): per particle of species s and corner c of its cell, with
// t = m_s W wcorr w_c, the ten sums rho = t, rho u = t v, rho u u = t v v
// (xx, yy, zz, xy, yz, xz), divided by the cell volume and summed on the
// corner.  Values are those of the particles after the step (the reference
// samples inside UpdateJMassMatrix, after the mover).
//
//   k_species_cells   one warp per cell, one pass per species present: every
//                     lane accumulates the 8 x 10 products of its particles
//                     in registers (FP32), the warp adds its 32 rows through
//                     shared memory; per-cell partials cellS[cell][s][10][8]
//   k_species_gather  FP64 corner sums over the cells that have the corner
//                     (a CSR built once per mesh), times 1 / cell volume;
//                     component-major out[(10 s + q) * ncorners + corner]
//
// Runs after the deposition when sampling is on (amps_gpu_set_species_moments);
// costs one more read of the particle state.
//
// Also here, on the same corner CSR:
//   k_amr_corner_moments  AMR contexts' J and M in the corner layout
//                     (amps_gpu_export_moments): one CTA per corner, FP32-pair
//                     sums of the cells' partials, written in corner ranges
//                     whose host copies overlap the next range's kernel
//   k_particle_cfl    the per-species maximum of ProcessCell's cflCell
//                     (amps_gpu_particle_cfl)
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "deposit_core.cuh"

namespace {

constexpr int kQ = 10;            // quantities per species (Rho_ .. RhoUxUz_)
constexpr int kV = 8 * kQ;        // values per species per cell
constexpr int kWarpsS = 4;        // 41.5 KB of static shared memory per CTA
constexpr int kRow = kV + 1;      // shared row stride (conflict-free columns)

struct SpecArgs {
  const float* u[3];
  const float* v[3];
  const uint8_t* sp;
  const float* wc;                // may be null
  const int* base;
  const int* cnt;
  long long ncell;
  int nspec;
  float mw[AMPS_GPU_MAX_SPECIES]; // m * W per species
  float* cellS;                   // [ncell][nspec][kQ][8]
};

__global__ void __launch_bounds__(kWarpsS * 32) k_species_cells(SpecArgs a) {
  __shared__ float red[kWarpsS][32 * kRow];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float* row = red[wid];
  const long long nw = (long long)gridDim.x * kWarpsS;
  for (long long cid = (long long)blockIdx.x * kWarpsS + wid; cid < a.ncell; cid += nw) {
    const int b0 = a.base[cid], n = a.cnt[cid];
    const int l = (int)(cid % AMPS_CPB);
    const float ci[3] = {(float)(l & 7), (float)((l >> 3) & 7), (float)(l >> 6)};
    unsigned present = 0;
    for (int q0 = lane; q0 < n; q0 += 32) present |= 1u << a.sp[b0 + q0];
    present = __reduce_or_sync(0xffffffffu, present);
    float* out = a.cellS + (size_t)cid * a.nspec * kV;
    for (int s = 0; s < a.nspec; s++) {
      if (!((present >> s) & 1u)) {
        for (int t = lane; t < kV; t += 32) out[s * kV + t] = 0.f;
        continue;
      }
      float acc[kV];
#pragma unroll
      for (int t = 0; t < kV; t++) acc[t] = 0.f;
      for (int q0 = lane; q0 < n; q0 += 32) {
        const int p = b0 + q0;
        if (a.sp[p] != s) continue;
        float f[3], vv[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          f[d] = a.u[d][p] - ci[d];
          vv[d] = a.v[d][p];
        }
        const float m = a.mw[s] * (a.wc ? a.wc[p] : 1.0f);
        const float val[kQ] = {m,
                               m * vv[0],
                               m * vv[1],
                               m * vv[2],
                               m * vv[0] * vv[0],
                               m * vv[1] * vv[1],
                               m * vv[2] * vv[2],
                               m * vv[0] * vv[1],
                               m * vv[1] * vv[2],
                               m * vv[0] * vv[2]};
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const float w = ((c & 1) ? f[0] : 1.f - f[0]) * ((c & 2) ? f[1] : 1.f - f[1]) *
                          ((c & 4) ? f[2] : 1.f - f[2]);
#pragma unroll
          for (int q = 0; q < kQ; q++) acc[q * 8 + c] = fmaf(w, val[q], acc[q * 8 + c]);
        }
      }
      // column sums of the warp's 32 rows
#pragma unroll
      for (int t = 0; t < kV; t++) row[lane * kRow + t] = acc[t];
      __syncwarp();
      for (int t = lane; t < kV; t += 32) {
        float sum = 0.f;
        for (int r = 0; r < 32; r++) sum += row[r * kRow + t];
        out[s * kV + t] = sum;
      }
      __syncwarp();
    }
  }
}

// out[(10 s + q) * nvc + corner] = sum over entries (cell, c) of the corner of
// cellS[cell][s][q][c] / V(cell)
__global__ void __launch_bounds__(256) k_species_gather(long long nvc, int nspec,
                                                        const int* __restrict__ start,
                                                        const int* __restrict__ ent,
                                                        const float* __restrict__ cellS,
                                                        const double* __restrict__ bdx,
                                                        double inv_vol, double* __restrict__ out) {
  const long long total = nvc * nspec * kQ;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long cc = t % nvc;
    const int k = (int)(t / nvc);  // 10 s + q
    double sum = 0.0;
    for (int e = start[cc]; e < start[cc + 1]; e++) {
      const int en = ent[e];
      const long long cell = en >> 3;
      const int c = en & 7;
      double iv = inv_vol;
      if (bdx) {
        const double dx = bdx[cell / AMPS_CPB];
        iv = 1.0 / (dx * dx * dx);
      }
      sum += (double)cellS[(size_t)cell * nspec * kV + (size_t)k * 8 + c] * iv;
    }
    out[t] = sum;
  }
}

}  // namespace

// Corner -> (cell, corner-of-cell) lists, built once per context.  Corner
// (i, j, k) of block b's cell grid (0..8 per axis) is the uniform lattice
// corner there (periodic), or the AMR mesh's unique corner from the block's
// corner table.  Entry = cell * 8 + q, q the corner's binary offset
// (q & 1, (q >> 1) & 1, q >> 2) in the cell.
amps_gpu_status corner_csr_setup(amps_gpu_ctx* c) {
  if (c->d_spec_start) return AMPS_GPU_OK;
  const long long nv = c->nvc;
  std::vector<int> ctab;
  if (c->amr) {
    ctab.resize((size_t)c->nb * 729);
    cudaError_t e = cudaMemcpy(ctab.data(), c->d_ctab, sizeof(int) * ctab.size(), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_check(c, e, "corner lists: corner table");
  }
  const int nbx = c->cfg.nbx, nby = c->cfg.nby, nbz = c->cfg.nbz;
  const int NX = 8 * nbx, NY = 8 * nby, NZ = 8 * nbz;
  auto corner = [&](int b, int ci, int cj, int ck) -> int {
    if (c->amr) return ctab[(size_t)b * 729 + ci + 9 * (cj + 9 * ck)];
    const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
    const int I = (8 * bx + ci) % NX, J = (8 * by + cj) % NY, K = (8 * bz + ck) % NZ;
    return ((I >> 3) + nbx * ((J >> 3) + nby * (K >> 3))) * AMPS_CPB + (I & 7) + 8 * ((J & 7) + 8 * (K & 7));
  };
  std::vector<int> count((size_t)nv + 1, 0);
  for (int b = 0; b < c->nb; b++)
    for (int l = 0; l < AMPS_CPB; l++)
      for (int q = 0; q < 8; q++)
        count[(size_t)corner(b, (l & 7) + (q & 1), ((l >> 3) & 7) + ((q >> 1) & 1), (l >> 6) + (q >> 2)) + 1]++;
  for (long long i = 0; i < nv; i++) count[(size_t)i + 1] += count[(size_t)i];
  std::vector<int> ent((size_t)count[(size_t)nv]), fill(count.begin(), count.end() - 1);
  for (int b = 0; b < c->nb; b++)
    for (int l = 0; l < AMPS_CPB; l++)
      for (int q = 0; q < 8; q++) {
        const int cc = corner(b, (l & 7) + (q & 1), ((l >> 3) & 7) + ((q >> 1) & 1), (l >> 6) + (q >> 2));
        ent[(size_t)fill[(size_t)cc]++] = (int)(((long long)b * AMPS_CPB + l) * 8 + q);
      }
  bool ok = cudaMalloc(reinterpret_cast<void**>(&c->d_spec_start), sizeof(int) * count.size()) == cudaSuccess &&
            cudaMalloc(reinterpret_cast<void**>(&c->d_spec_ent), sizeof(int) * std::max<size_t>(ent.size(), 1)) == cudaSuccess;
  ok = ok && cudaMemcpy(c->d_spec_start, count.data(), sizeof(int) * count.size(), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(c->d_spec_ent, ent.data(), sizeof(int) * ent.size(), cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    cudaFree(c->d_spec_start);
    cudaFree(c->d_spec_ent);
    c->d_spec_start = c->d_spec_ent = nullptr;
    return set_err(c, AMPS_GPU_CUDA_ERROR, "corner lists: allocation failed");
  }
  return AMPS_GPU_OK;
}

amps_gpu_status species_setup(amps_gpu_ctx* c, bool on) {
  if (!on) {
    c->spec_on = false;
    return AMPS_GPU_OK;
  }
  amps_gpu_status st = corner_csr_setup(c);
  if (st) return st;
  if (!c->d_cellS) {
    const long long nv = c->nvc;
    bool ok = cudaMalloc(reinterpret_cast<void**>(&c->d_cellS),
                         sizeof(float) * (size_t)c->ncor * c->cfg.nspec * kV) == cudaSuccess &&
              cudaMalloc(reinterpret_cast<void**>(&c->d_specC),
                         sizeof(double) * (size_t)nv * c->cfg.nspec * kQ) == cudaSuccess;
    ok = ok && cudaMemset(c->d_specC, 0, sizeof(double) * (size_t)nv * c->cfg.nspec * kQ) == cudaSuccess;
    if (!ok) {
      cudaGetLastError();
      species_free(c);
      return set_err(c, AMPS_GPU_CUDA_ERROR, "species moments: allocation failed");
    }
  }
  c->spec_on = true;
  return AMPS_GPU_OK;
}

void species_free(amps_gpu_ctx* c) {
  cudaFree(c->d_bivh);
  c->d_bivh = nullptr;
  cudaFree(c->d_amrJ);
  cudaFree(c->d_amrM);
  c->d_amrJ = c->d_amrM = nullptr;
  cudaFree(c->d_cellS);
  cudaFree(c->d_specC);
  cudaFree(c->d_spec_start);
  cudaFree(c->d_spec_ent);
  c->d_cellS = nullptr;
  c->d_specC = nullptr;
  c->d_spec_start = c->d_spec_ent = nullptr;
  c->spec_on = false;
}

cudaError_t launch_species_moments(amps_gpu_ctx* c) {
  if (!c->spec_on) return cudaSuccess;
  SpecArgs a{};
  for (int d = 0; d < 3; d++) {
    a.u[d] = c->d_u[c->cur][d];
    a.v[d] = c->d_v[c->cur][d];
  }
  a.sp = c->d_sp[c->cur];
  a.wc = c->has_wcorr ? c->d_wc[c->cur] : nullptr;
  a.base = c->d_base;
  a.cnt = c->d_cnt;
  a.ncell = c->ncor;
  a.nspec = c->cfg.nspec;
  for (int s = 0; s < c->cfg.nspec; s++) a.mw[s] = (float)(c->cfg.mass[s] * c->cfg.weight[s]);
  a.cellS = c->d_cellS;
  {
    TimedLaunch t(c, "species_cells");
    const long long blocks = std::min<long long>((c->ncor + kWarpsS - 1) / kWarpsS, 152LL * 16);
    k_species_cells<<<(unsigned)blocks, kWarpsS * 32, 0, c->stream>>>(a);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  {
    TimedLaunch t(c, "species_gather");
    const double V = c->cfg.dx[0] * c->cfg.dx[1] * c->cfg.dx[2];
    const long long total = c->nvc * c->cfg.nspec * kQ;
    const long long blocks = std::min<long long>((total + 255) / 256, 152LL * 32);
    k_species_gather<<<(unsigned)blocks, 256, 0, c->stream>>>(
        c->nvc, c->cfg.nspec, c->d_spec_start, c->d_spec_ent, c->d_cellS,
        c->amr ? c->d_bdx : nullptr, 1.0 / V, c->d_specC);
  }
  return cudaGetLastError();
}

// Per-species CFL number of UpdateJMassMatrix (ProcessCell,
// src/pic/pic_field_solver_ecsim.cpp:2236 and :2356-2359; maximum over cells
// :3352, :3972-3977): per cell and species the mean particle speed times dt
// over the cell diagonal, maximum over the cells holding that species.  One
// warp per cell, one pass per species present; |v| as a float pair (exact
// squares, TwoSum, sqrt with one Newton correction), cell sums as float
// pairs, the ratio in FP64 by one lane; the maximum by an integer atomicMax on
// the bits of a non-negative double.
struct CflArgs {
  const float* v[3];
  const uint8_t* sp;
  const int* base;
  const int* cnt;
  long long ncell;
  int nspec;
  double dt;
  double diag;                 // uniform meshes: |(dx, dy, dz)|
  const double* bdx;           // AMR meshes: cell size per block (diagonal sqrt(3) dx)
  unsigned long long* cfl;     // [nspec] bits of the FP64 maximum
};

__device__ __forceinline__ FF speed_ff(float v0, float v1, float v2) {
  const float p0 = __fmul_rn(v0, v0);
  FF t{p0, fmaf(v0, v0, -p0)};
  ff_add(t, v1, v1, 0.f);
  ff_add(t, v2, v2, 0.f);
  t = ff_norm(t);
  const float r = __fsqrt_rn(t.s);
  if (r == 0.f) return FF{0.f, 0.f};
  // sqrt(s + q) = r + (s - r^2 + q) / (2 r) to second order; s - r^2 is exact
  const float e = __fadd_rn(fmaf(-r, r, t.s), t.q);
  return FF{r, __fdiv_rn(e, __fmul_rn(2.f, r))};
}

__global__ void __launch_bounds__(256) k_particle_cfl(CflArgs a) {
  const int lane = threadIdx.x & 31;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long cid = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); cid < a.ncell;
       cid += nw) {
    const int b0 = a.base[cid], n = a.cnt[cid];
    unsigned present = 0;
    for (int q = lane; q < n; q += 32) present |= 1u << a.sp[b0 + q];
    present = __reduce_or_sync(0xffffffffu, present);
    for (int s = 0; s < a.nspec; s++) {
      if (!((present >> s) & 1u)) continue;
      FF sum{0.f, 0.f};
      int count = 0;
      for (int q = lane; q < n; q += 32) {
        const int p = b0 + q;
        if (a.sp[p] != s) continue;
        const FF sv = speed_ff(a.v[0][p], a.v[1][p], a.v[2][p]);
        ff_acc(sum, sv.s, sv.q);
        count++;
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float hs = __shfl_xor_sync(0xffffffffu, sum.s, o);
        const float hq = __shfl_xor_sync(0xffffffffu, sum.q, o);
        ff_acc(sum, hs, hq);
        count += __shfl_xor_sync(0xffffffffu, count, o);
      }
      if (lane == 0 && count > 0) {
        const double diag = a.bdx ? 1.7320508075688772 * a.bdx[cid / AMPS_CPB] : a.diag;
        const double cfl = ff_value(sum) * a.dt / ((double)count * diag);
        atomicMax(a.cfl + s, (unsigned long long)__double_as_longlong(cfl));
      }
    }
  }
}

// AMR moments in the corner layout: what ProcessCell's flush
// (pic_field_solver_ecsim.cpp:2362-2426) adds into the corner nodes, summed
// over the cells (of any level) that have the corner -- J[corner][3] =
// sum cellJ / V(cell), M[corner][27 slots][9] with slot(d) = dig(dx) +
// 3 dig(dy) + 9 dig(dz), dig(0) = 0, dig(-1) = 1, dig(+1) = 2, d the partner
// corner's offset in the cell (IndexMatrix, :1889-1891) and the block the
// cell's partial of the pair's weight monomial (already divided by V).  One
// CTA per corner: thread t < 243 sums M element t over the corner's cells (in
// CSR order, the cells whose pair lies inside them), threads 243..245 the J
// components; the cells' entries are staged in shared memory first, so the
// loads of the partials of all the corner's cells are independent.  The sums
// are FP32 pairs (error-free TwoSum; J's 1/V an FP32 pair per block, ivh/ivl)
// widened once: a warp-wide FP64 instruction occupies GB300's narrow FP64
// pipe ~64x longer than an FP32 one, and FP64 adds and divides made this
// kernel 8.6 ms per export of config 2.  Hanging corners get their own sums.
// Corners [c0, c1); J or M may be null.
constexpr int kCmThreads = 256;
constexpr int kCmEnt = 32;  // entries staged per corner (more are read from global memory)
__global__ void __launch_bounds__(kCmThreads) k_amr_corner_moments(
    long long c0, long long c1, const int* __restrict__ start, const int* __restrict__ ent,
    const float* __restrict__ cellM, const float* __restrict__ cellJ, const float* __restrict__ ivh,
    const float* __restrict__ ivl, double* __restrict__ J, double* __restrict__ M) {
  __shared__ int s_ent[kCmEnt];
  __shared__ int s_rng[2];
  const int t = threadIdx.x;
  // this thread's M element: slot t / 9 (digits 0, 1, 2 = offsets 0, -1, +1), component t % 9
  const int slot = t / 9, comp = t - 9 * slot;
  const int dg[3] = {slot % 3, (slot / 3) % 3, slot / 9};
  int d[3];
#pragma unroll
  for (int a = 0; a < 3; a++) d[a] = dg[a] == 0 ? 0 : (dg[a] == 1 ? -1 : 1);
  for (long long cc = c0 + blockIdx.x; cc < c1; cc += gridDim.x) {
    if (t == 0) {
      s_rng[0] = start[cc];
      s_rng[1] = start[cc + 1];
    }
    __syncthreads();
    const int e0 = s_rng[0], ne = s_rng[1] - s_rng[0];
    if (t < ne && t < kCmEnt) s_ent[t] = ent[e0 + t];
    __syncthreads();
    FF sum{0.f, 0.f};
    if (t < 243) {
      if (M) {
#pragma unroll 4
        for (int e = 0; e < ne; e++) {
          const int en = e < kCmEnt ? s_ent[e] : ent[e0 + e];
          const int q = en & 7;  // the corner's offset bits in the cell (x, y, z)
          const int o0 = (q & 1) + d[0], o1 = ((q >> 1) & 1) + d[1], o2 = (q >> 2) + d[2];
          if ((unsigned)o0 > 1u || (unsigned)o1 > 1u || (unsigned)o2 > 1u) continue;
          const int mono = ((q & 1) + o0) + 3 * (((q >> 1) & 1) + o1) + 9 * ((q >> 2) + o2);
          ff_acc(sum, cellM[cellM_at(en >> 3, mono * 9 + comp)], 0.f);
        }
        M[cc * 243 + t] = widen(sum.s) + widen(sum.q);
      }
    } else if (t < 246 && J) {
      const int jc = t - 243;
      for (int e = 0; e < ne; e++) {
        const int en = e < kCmEnt ? s_ent[e] : ent[e0 + e];
        const long long cell = en >> 3;
        const int q = en & 7, b = (int)(cell / AMPS_CPB);
        const FF p = ff_mul(cellJ[cellJ_at(cell, (q ^ ((q >> 1) & 1)) * 3 + jc)], 0.f, ivh[b], ivl[b]);
        ff_acc(sum, p.s, p.q);
      }
      J[cc * 3 + jc] = widen(sum.s) + widen(sum.q);
    }
    __syncthreads();  // s_rng and s_ent are rewritten for the next corner
  }
}

// the corner-layout moments of an AMR context (k_amr_corner_moments) into
// host J[nvc][3], M[nvc][243] (mesh corner numbering).  The kernel writes a
// device buffer in kCmChunks corner ranges; each range's copy to the host
// runs on the copy stream while the kernel produces the next, so a
// page-locked destination fills at the host link's rate.
constexpr int kCmChunks = 16;
static_assert(sizeof(amps_gpu_ctx::copy_ev) / sizeof(cudaEvent_t) >= kCmChunks + 1,
              "one event per export chunk and one for the end");
amps_gpu_status amr_export_corner_moments(amps_gpu_ctx* c, double* J, double* M) {
  amps_gpu_status st = corner_csr_setup(c);
  if (st) return st;
  if (!J && !M) return AMPS_GPU_OK;
  if (!c->d_amrJ) {
    if (cudaMalloc(reinterpret_cast<void**>(&c->d_amrJ), sizeof(double) * 3 * (size_t)c->nvc) != cudaSuccess ||
        cudaMalloc(reinterpret_cast<void**>(&c->d_amrM), sizeof(double) * 243 * (size_t)c->nvc) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(c->d_amrJ);
      c->d_amrJ = nullptr;
      return set_err(c, AMPS_GPU_CUDA_ERROR, "export_moments: allocation failed");
    }
  }
  if (!c->d_bivh) {
    // 1/dx^3 per block as an FP32 pair
    std::vector<double> bdx((size_t)c->nb);
    if ((st = cuda_check(c, cudaMemcpy(bdx.data(), c->d_bdx, sizeof(double) * bdx.size(),
                                       cudaMemcpyDeviceToHost), "block sizes")))
      return st;
    std::vector<float> iv(2 * bdx.size());
    for (size_t b = 0; b < bdx.size(); b++) {
      const double v = 1.0 / (bdx[b] * bdx[b] * bdx[b]);
      iv[b] = (float)v;
      iv[bdx.size() + b] = (float)(v - (double)iv[b]);
    }
    if (cudaMalloc(reinterpret_cast<void**>(&c->d_bivh), sizeof(float) * iv.size()) != cudaSuccess) {
      cudaGetLastError();
      c->d_bivh = nullptr;
      return set_err(c, AMPS_GPU_CUDA_ERROR, "export_moments: allocation failed");
    }
    if ((st = cuda_check(c, cudaMemcpy(c->d_bivh, iv.data(), sizeof(float) * iv.size(),
                                       cudaMemcpyHostToDevice), "block volumes")))
      return st;
  }
  if (!c->copy_stream) {
    if ((st = cuda_check(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking),
                         "copy stream")))
      return st;
    for (auto& e : c->copy_ev)
      if ((st = cuda_check(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "copy event")))
        return st;
  }
  const long long per = (c->nvc + kCmChunks - 1) / kCmChunks;
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < kCmChunks && e == cudaSuccess; k++) {
    const long long a = std::min<long long>(c->nvc, k * per), b = std::min<long long>(c->nvc, a + per);
    if (a >= b) break;
    {
      TimedLaunch t(c, "amr_corner_moments");
      const long long blocks = std::min<long long>(b - a, 152LL * 8);
      k_amr_corner_moments<<<(unsigned)blocks, kCmThreads, 0, c->stream>>>(
          a, b, c->d_spec_start, c->d_spec_ent, c->d_cellM, c->d_cellJ, c->d_bivh, c->d_bivh + c->nb,
          J ? c->d_amrJ : nullptr, M ? c->d_amrM : nullptr);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventRecord(c->copy_ev[k], c->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->copy_stream, c->copy_ev[k], 0);
    if (e == cudaSuccess && M)
      e = cudaMemcpyAsync(M + a * 243, c->d_amrM + a * 243, sizeof(double) * 243 * (size_t)(b - a),
                          cudaMemcpyDeviceToHost, c->copy_stream);
    if (e == cudaSuccess && J)
      e = cudaMemcpyAsync(J + a * 3, c->d_amrJ + a * 3, sizeof(double) * 3 * (size_t)(b - a),
                          cudaMemcpyDeviceToHost, c->copy_stream);
  }
  // the context's stream resumes after the last copy
  if (e == cudaSuccess) e = cudaEventRecord(c->copy_ev[kCmChunks], c->copy_stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->stream, c->copy_ev[kCmChunks], 0);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_check(c, e, "export corner moments");
}

extern "C" {

amps_gpu_status amps_gpu_particle_cfl(amps_gpu_ctx* c, double* cfl) {
  if (!c || !cfl) return set_err(c, AMPS_GPU_INVALID_ARG, "particle_cfl: null output");
  cudaSetDevice(c->cfg.device);
  CflArgs a{};
  for (int d = 0; d < 3; d++) a.v[d] = c->d_v[c->cur][d];
  a.sp = c->d_sp[c->cur];
  a.base = c->d_base;
  a.cnt = c->d_cnt;
  a.ncell = c->ncor;
  a.nspec = c->cfg.nspec;
  a.dt = c->cfg.dt;
  a.diag = sqrt(c->cfg.dx[0] * c->cfg.dx[0] + c->cfg.dx[1] * c->cfg.dx[1] +
                c->cfg.dx[2] * c->cfg.dx[2]);
  a.bdx = c->amr ? c->d_bdx : nullptr;
  a.cfl = reinterpret_cast<unsigned long long*>(c->d_energy + 4);
  amps_gpu_status st;
  if ((st = cuda_check(c, cudaMemsetAsync(a.cfl, 0, AMPS_GPU_MAX_SPECIES * sizeof(double), c->stream),
                       "cfl reset")))
    return st;
  {
    TimedLaunch t(c, "particle_cfl");
    const long long blocks = std::min<long long>((c->ncor + 7) / 8, 152LL * 16);
    if (blocks > 0) k_particle_cfl<<<(unsigned)blocks, 256, 0, c->stream>>>(a);
  }
  if ((st = cuda_check(c, cudaGetLastError(), "particle_cfl"))) return st;
  double out[AMPS_GPU_MAX_SPECIES];
  if ((st = cuda_check(c, cudaMemcpyAsync(out, c->d_energy + 4, c->cfg.nspec * sizeof(double),
                                          cudaMemcpyDeviceToHost, c->stream), "cfl")))
    return st;
  if ((st = cuda_check(c, cudaStreamSynchronize(c->stream), "sync"))) return st;
  for (int s = 0; s < c->cfg.nspec; s++) cfl[s] = out[s];
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_set_species_moments(amps_gpu_ctx* c, int on) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  cudaStreamSynchronize(c->stream);
  return species_setup(c, on != 0);
}

amps_gpu_status amps_gpu_export_species_moments(amps_gpu_ctx* c, double* out) {
  if (!c || !out) return set_err(c, AMPS_GPU_INVALID_ARG, "export_species_moments: null output");
  if (!c->d_specC)
    return set_err(c, AMPS_GPU_INVALID_ARG, "export_species_moments: sampling was never switched on");
  cudaSetDevice(c->cfg.device);
  return layout_download(c, c->d_specC, out, c->nvc, c->cfg.nspec * kQ, false);
}

}  // extern "C"
