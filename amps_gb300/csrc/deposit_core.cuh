// Device code shared by the particle kernels (particles.cu) and the
// no-allocation deposition entry point (noalloc.cu): species constants, the
// bulk-copy staging of block stencils, the per-particle deposition fields,
// the register-tile accumulation (packed FP32x2 FMAs) with FP32 chunk sums,
// and FP32 -> FP64 widening.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "ptx.cuh"

namespace {
constexpr uint32_t kWaitLimit = 1u << 24;
// Staged deposition fields, a structure of arrays per warp: field f of the
// record at position p is rec[f * FS + p].  A chunk stages one record per
// lane (position = lane); particles that do not deposit stage zero weight.
//   0..26  the 27 trilinear weight monomials X_x[a] X_y[b] X_z[c], a + 3b + 9c
//   27..35 k alpha, row-major 3x3, k = q W h / V
//   36..43 the 8 corner weights
//   44     zero (pads the last current lane's third weight)
//   45..47 q W alpha v
// FS is the positions per field plus 4, so the 16-byte loads of 4 positions
// of different fields spread over the banks and the per-lane stores of one
// field are conflict-free.
constexpr int kFields = 48;
constexpr int kFS = 36;       // 32-position chunks (push/deposit, full deposit)
constexpr int kTileLanes = 30;  // lanes owning a 3 x 3 output tile
constexpr int kWarps = 8;     // warps per CTA (one row of 8 cells each)
constexpr uint8_t kHole = 0xFF;

struct SpeciesTab {
  float qdt2m[AMPS_GPU_MAX_SPECIES];  // 0.5*q*dt/m (weight independent)
  float qw[AMPS_GPU_MAX_SPECIES];     // q*w
  float keh[AMPS_GPU_MAX_SPECIES];    // 0.5*m*w (FP64) = keh + kel, two floats
  float kel[AMPS_GPU_MAX_SPECIES];
};

SpeciesTab make_species(const amps_gpu_config& c) {
  SpeciesTab t{};
  for (int s = 0; s < c.nspec; s++) {
    t.qdt2m[s] = (float)(0.5 * (c.charge[s] * c.dt / c.mass[s]));
    t.qw[s] = (float)(c.charge[s] * c.weight[s]);
    const double ke = 0.5 * c.mass[s] * c.weight[s];
    t.keh[s] = (float)ke;
    t.kel[s] = (float)(ke - (double)t.keh[s]);
  }
  return t;
}

// en += the kinetic energy 0.5 m W v^2 of one particle (ProcessCell :2238,
// summed in FP64 by the reference) as a float pair: the squares and the
// weight-correction product exact by FMA, sums by TwoSum, the FP64 species
// factor 0.5 m w as two floats (FF, common.cuh).  Error ~1e-14 of the sum.
__device__ __forceinline__ void kinetic_energy(FF& en, float v0, float v1, float v2, float wcorr,
                                               int s, const SpeciesTab& st) {
  const float p0 = __fmul_rn(v0, v0);
  FF t{p0, fmaf(v0, v0, -p0)};
  ff_add(t, v1, v1, 0.f);
  ff_add(t, v2, v2, 0.f);
  const FF tw = ff_mul(t.s, t.q, wcorr, 0.f);
  ff_add2(en, st.keh[s], st.kel[s], tw.s, tw.q);
}

// Stage one bulk copy per stencil into shared memory; returns false on timeout.
__device__ bool stage_stencils(uint64_t* bar, void* dst0, const void* src0, uint32_t bytes0,
                               void* dst1, const void* src1, uint32_t bytes1,
                               unsigned long long* flags, void* dst2 = nullptr,
                               const void* src2 = nullptr, uint32_t bytes2 = 0) {
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(bar, bytes0 + bytes1 + bytes2);
    if (bytes0) bulk_copy_g2s(dst0, src0, bytes0, bar);
    if (bytes1) bulk_copy_g2s(dst1, src1, bytes1, bar);
    if (bytes2) bulk_copy_g2s(dst2, src2, bytes2, bar);
  }
  if (!mbar_wait_bounded(bar, 0, kWaitLimit)) {
    if (threadIdx.x == 0) atomicAdd(flags + 2, 1ull);
    mbar_wait_bounded(bar, 0, kWaitLimit);  // let the copies land before exiting
    return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Deposition pieces shared by k_push_deposit, k_arrivals and k_deposit.

// Per-cell partial sums, contiguous per cell.  Mass matrix: the product of two
// trilinear corner weights depends only on the per-axis sums a_d = o1_d + o2_d
// of the corners' offsets, w_c1 w_c2 = X_x[a_x] X_y[a_y] X_z[a_z] with
// X[0] = (1-f)^2, X[1] = f(1-f), X[2] = f^2, so ProcessCell's 36 corner-pair
// blocks are 27 distinct monomial sums x 9 (index (a_x + 3 a_y + 9 a_z) * 9 +
// row * 3 + col).  Current: 8 corners x 3.
__host__ __device__ __forceinline__ long long cellM_at(long long cid, int pe) {
  return cid * AMPS_CELLM + pe;
}
// monomial index of the corner pair (c1, c2) in the table order of the corners
__host__ __device__ __forceinline__ int pair_monomial(int c1, int c2) {
  const int ox[8] = {0, 1, 1, 0, 0, 1, 1, 0}, oy[8] = {0, 0, 1, 1, 0, 0, 1, 1},
            oz[8] = {0, 0, 0, 0, 1, 1, 1, 1};
  return (ox[c1] + ox[c2]) + 3 * (oy[c1] + oy[c2]) + 9 * (oz[c1] + oz[c2]);
}
__host__ __device__ __forceinline__ long long cellJ_at(long long cid, int ce) {
  return cid * 24 + ce;
}

// B at block-local offset u from a centre stencil (10^3 cell centres of the
// block incl. the +-1 halo): CellCentered::Linear's trilinear weights
// (pic_interpolation_routines.cpp:820-905: i0 = -1 below half a cell, else
// (int)(u - 0.5), weight u - (i0 + 0.5))
__device__ __forceinline__ void centre_b(const float4* __restrict__ sC, float u0, float u1, float u2,
                                         float B[3]) {
  const float u[3] = {u0, u1, u2};
  int o[3];
  float w[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    o[d] = u[d] < 0.5f ? -1 : (int)(u[d] - 0.5f);
    w[d] = u[d] - ((float)o[d] + 0.5f);
  }
  const int s0 = (o[0] + 1) + 10 * ((o[1] + 1) + 10 * (o[2] + 1));
  float Bs[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
  for (int c = 0; c < 2; c++)
#pragma unroll
    for (int b = 0; b < 2; b++)
#pragma unroll
      for (int a = 0; a < 2; a++) {
        const float W = (a ? w[0] : 1.f - w[0]) * (b ? w[1] : 1.f - w[1]) * (c ? w[2] : 1.f - w[2]);
        const float4 q = sC[s0 + a + 10 * b + 100 * c];
        Bs[c][0] = fmaf(W, q.x, Bs[c][0]);
        Bs[c][1] = fmaf(W, q.y, Bs[c][1]);
        Bs[c][2] = fmaf(W, q.z, Bs[c][2]);
      }
  B[0] = Bs[0][0] + Bs[1][0];
  B[1] = Bs[0][1] + Bs[1][1];
  B[2] = Bs[0][2] + Bs[1][2];
}

// The fields of one particle at block-local offset u inside cell (i,j,k), at
// record position pos; wq = q weight correction of a depositing particle, 0
// for a lane that deposits nothing (its k alpha and q alpha v, hence all its
// products, are zero).  Adds its kinetic energy (weighted by wq) to en.  sB:
// the corner B stencil, or (CB) the centre B stencil.
template <int FS, bool CB = false>
__device__ __forceinline__ void stage_fields(float* __restrict__ rec, int pos,
                                             const float4* __restrict__ sB, float u0, float u1,
                                             float u2, float v0, float v1, float v2, int s,
                                             float wq, int i, int j, int k,
                                             const SpeciesTab& st, float inv_vol, FF& en) {
  const float fx = fminf(fmaxf(u0 - (float)i, 0.f), 1.f);
  const float fy = fminf(fmaxf(u1 - (float)j, 0.f), 1.f);
  const float fz = fminf(fmaxf(u2 - (float)k, 0.f), 1.f);
  const float gx = 1.f - fx, gy = 1.f - fy, gz = 1.f - fz;
  float w[8];
  w[0] = gx * gy * gz; w[1] = fx * gy * gz; w[2] = fx * fy * gz; w[3] = gx * fy * gz;
  w[4] = gx * gy * fz; w[5] = fx * gy * fz; w[6] = fx * fy * fz; w[7] = gx * fy * fz;
  float B0, B1, B2;
  if (CB) {
    float Bc[3];
    centre_b(sB, u0, u1, u2, Bc);
    B0 = Bc[0];
    B1 = Bc[1];
    B2 = Bc[2];
  } else {
    const int sb = i + 9 * (j + 9 * k);
    const int coff[8] = {0, 1, 10, 9, 81, 82, 91, 90};
    // two partial sums per component (corners 0-3, 4-7): six independent chains
    float Bs[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const float4 q = sB[sb + coff[c]];
      Bs[c >> 2][0] = fmaf(w[c], q.x, Bs[c >> 2][0]);
      Bs[c >> 2][1] = fmaf(w[c], q.y, Bs[c >> 2][1]);
      Bs[c >> 2][2] = fmaf(w[c], q.z, Bs[c >> 2][2]);
    }
    B0 = Bs[0][0] + Bs[1][0];
    B1 = Bs[0][1] + Bs[1][1];
    B2 = Bs[0][2] + Bs[1][2];
  }
  const float h = st.qdt2m[s];
  const float h2 = h * h;
  const float c0 = 1.0f / (1.0f + h2 * (B0 * B0 + B1 * B1 + B2 * B2));
  const float P0 = -h * B0, P1 = -h * B1, P2 = -h * B2;
  float al[9];
  al[0] = c0 * (1.f + h2 * B0 * B0);
  al[1] = c0 * (-P2 + h2 * B0 * B1);
  al[2] = c0 * (P1 + h2 * B0 * B2);
  al[3] = c0 * (P2 + h2 * B1 * B0);
  al[4] = c0 * (1.f + h2 * B1 * B1);
  al[5] = c0 * (-P0 + h2 * B1 * B2);
  al[6] = c0 * (-P1 + h2 * B2 * B0);
  al[7] = c0 * (P0 + h2 * B2 * B1);
  al[8] = c0 * (1.f + h2 * B2 * B2);
  const float qW = st.qw[s] * wq;
  const float kc = qW * h * inv_vol;
  float* r = rec + pos;
  {
    const float X[3] = {gx * gx, gx * fx, fx * fx};
    const float Y[3] = {gy * gy, gy * fy, fy * fy};
    const float Z[3] = {gz * gz, gz * fz, fz * fz};
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
      for (int b = 0; b < 3; b++) {
        const float yz = Y[b] * Z[c];
#pragma unroll
        for (int a = 0; a < 3; a++) r[(a + 3 * b + 9 * c) * FS] = X[a] * yz;
      }
  }
#pragma unroll
  for (int e = 0; e < 9; e++) r[(27 + e) * FS] = kc * al[e];
#pragma unroll
  for (int c = 0; c < 8; c++) r[(36 + c) * FS] = w[c];
  r[44 * FS] = 0.f;
  const float vr0 = al[0] * v0 + al[1] * v1 + al[2] * v2;
  const float vr1 = al[3] * v0 + al[4] * v1 + al[5] * v2;
  const float vr2 = al[6] * v0 + al[7] * v1 + al[8] * v2;
  r[45 * FS] = qW * vr0;
  r[46 * FS] = qW * vr1;
  r[47 * FS] = qW * vr2;
  kinetic_energy(en, v0, v1, v2, wq, s, st);
}

// d += a * b on packed FP32 pairs (two independent FMAs per instruction)
__device__ __forceinline__ void ffma2(unsigned long long& d, unsigned long long a,
                                      unsigned long long b) {
  asm("fma.rn.f32x2 %0, %1, %2, %0;" : "+l"(d) : "l"(a), "l"(b));
}

// Each of the first kTileLanes lanes owns a 3 x 3 tile: lanes 0..26 the
// products (monomials 3g..3g+2) x (k alpha row hh), lanes 27..29 the products
// (corner weights 3g'..3g'+2) x (q W alpha v); lanes 30, 31 repeat lane 27's
// loads and discard the result.  Four records cost every lane six 16-byte
// shared loads (4 positions of each of its 3 + 3 fields) and 18 packed FMAs,
// the even and odd positions accumulated in the two halves of each pair.
struct Tile {
  float sum[9];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int e = 0; e < 9; e++) sum[e] = 0.f;
  }
  // accumulate the staged positions [0, npos) (npos a multiple of 4) and add
  // the chunk's sums.  A Kahan-compensated add here changed the full-size
  // per-cell J and M errors against the FP64 oracle in no printed digit
  // (4.6e-7, 1.0e-6 at 128 particles per cell; the FP32 positions dominate)
  // and cost 4 % of the push/deposit kernel's time.
  template <int FS>
  __device__ __forceinline__ void accumulate(const float* __restrict__ rec, int npos, int fA,
                                             int fB) {
    unsigned long long acc[9];
#pragma unroll
    for (int e = 0; e < 9; e++) acc[e] = 0ull;
    const float* pa = rec + fA * FS;
    const float* pb = rec + fB * FS;
    // four staged positions: six 16-byte loads, 18 packed FMAs -- the 9
    // positions-(r, r+1) products first, then the 9 (r+2, r+3) ones: 9
    // independent accumulators between dependent packed FMAs
    auto four = [&](int r) {
      ulonglong2 A[3], B[3];
#pragma unroll
      for (int q = 0; q < 3; q++) {
        A[q] = *reinterpret_cast<const ulonglong2*>(pa + q * FS + r);
        B[q] = *reinterpret_cast<const ulonglong2*>(pb + q * FS + r);
      }
#pragma unroll
      for (int q = 0; q < 3; q++)
#pragma unroll
        for (int e = 0; e < 3; e++) ffma2(acc[3 * q + e], A[q].x, B[e].x);
#pragma unroll
      for (int q = 0; q < 3; q++)
#pragma unroll
        for (int e = 0; e < 3; e++) ffma2(acc[3 * q + e], A[q].y, B[e].y);
    };
    if (npos == FS - 4) {
      // a full chunk: no loop control
#pragma unroll
      for (int r = 0; r < FS - 4; r += 4) four(r);
    } else {
#pragma unroll 2
      for (int r = 0; r < npos; r += 4) four(r);
    }
#pragma unroll
    for (int e = 0; e < 9; e++) {
      const float2 a = *reinterpret_cast<const float2*>(&acc[e]);
      sum[e] += a.x + a.y;
    }
  }
  // write the tile's sums to the cell partials
  __device__ __forceinline__ void flush(int lane, float* __restrict__ cellM,
                                        float* __restrict__ cellJ, long long cid) const {
    if (lane < 27) {
      const int g = lane / 3, hh = lane % 3;
#pragma unroll
      for (int q = 0; q < 3; q++)
#pragma unroll
        for (int e = 0; e < 3; e++)
          cellM[cellM_at(cid, (3 * g + q) * 9 + 3 * hh + e)] = sum[3 * q + e];
    } else if (lane < kTileLanes) {
      const int g = lane - 27;
#pragma unroll
      for (int q = 0; q < 3; q++)
        if (3 * g + q < 8)
#pragma unroll
          for (int e = 0; e < 3; e++)
            cellJ[cellJ_at(cid, (3 * g + q) * 3 + e)] = sum[3 * q + e];
    }
  }
  // add the tile's sums to the cell partials by global reductions, which the
  // L2 performs without a read-back in the warp.  The warp first parks its 267
  // sums in scr at their partial offsets, so every reduction then covers 32
  // consecutive partials (4 sectors) instead of one partial in each of ~28
  // sectors: the L2's sector rate bounds a reduction-heavy pass.  scr is the
  // warp's staging area; the caller's accumulates are complete (__syncwarp).
  __device__ __forceinline__ void flush_red(int lane, float* __restrict__ scr,
                                            float* __restrict__ cellM,
                                            float* __restrict__ cellJ, long long cid) const {
    if (lane < 27) {
      const int g = lane / 3, hh = lane % 3;
#pragma unroll
      for (int q = 0; q < 3; q++)
#pragma unroll
        for (int e = 0; e < 3; e++) scr[(3 * g + q) * 9 + 3 * hh + e] = sum[3 * q + e];
    } else if (lane < kTileLanes) {
      const int g = lane - 27;
#pragma unroll
      for (int q = 0; q < 3; q++)
        if (3 * g + q < 8)
#pragma unroll
          for (int e = 0; e < 3; e++)
            scr[AMPS_CELLM + (3 * g + q) * 3 + e] = sum[3 * q + e];
    }
    __syncwarp();
    float* m = cellM + cellM_at(cid, 0);
#pragma unroll
    for (int r = 0; r < (AMPS_CELLM + 31) / 32; r++) {
      const int t = lane + 32 * r;
      if (t < AMPS_CELLM) atomicAdd(m + t, scr[t]);
    }
    if (lane < 24) atomicAdd(cellJ + cellJ_at(cid, lane), scr[AMPS_CELLM + lane]);
    __syncwarp();
  }
};

// the first A field and the first B field of this lane's tile
__device__ __forceinline__ void lane_fields(int lane, int& fA, int& fB) {
  if (lane < 27) {
    fA = 3 * (lane / 3);
    fB = 27 + 3 * (lane % 3);
  } else {
    fA = 36 + 3 * (lane < kTileLanes ? lane - 27 : 0);
    fB = 45;
  }
}

__device__ __forceinline__ void reduce_energy(double en, double* s_en, double* energy) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) en += __shfl_xor_sync(0xffffffffu, en, o);
  if ((threadIdx.x & 31) == 0) s_en[threadIdx.x >> 5] = en;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_en[w];
    if (t != 0.0) atomicAdd(energy, t);
  }
}

}  // namespace
