// Particle kernels of the ECSIM hot path on sm_103a.
//
//   k_pack_stencils  per-block FP32 copies of E^{n+theta}, corner B^n, corner
//                    B^{n+1} on the block's 9^3 corners (the SetBlock_E/SetBlock_B
//                    scratch of src/pic/pic_mover.cpp:86-167)
//   k_push           Lapenta2017 (src/pic/pic_mover_boris.cpp:876-1120) +
//                    destination block/cell (findTreeNode/FindCellIndex,
//                    meshAMRgeneric.h:2256-2320,2852-2883) with periodic wrap
//                    (pic_bc_periodic.cpp:86-178); warp-aggregated cell counts
//   k_scan_*         exclusive scan of the per-cell counts
//   k_scatter        stable-by-warp scatter into the destination cell ranges
//                    (the temp-list commit of pic_mover.cpp:982-1087)
//   k_deposit        ProcessCell (pic_field_solver_ecsim.cpp:1882-2438): one warp
//                    per cell, FP32 per-particle terms, register tiles, Kahan-
//                    compensated chunk sums, per-cell partials
//   k_assemble       flush of the per-cell partials into the 243-term corner
//                    mass matrix and corner J (:2362-2426 and the shared-corner
//                    sum of :3931-3968), FP64
#include <cuda_runtime.h>

#include <cstdio>

#include "common.cuh"
#include "ptx.cuh"

namespace {

constexpr uint32_t kWaitLimit = 1u << 24;

struct SpeciesTab {
  float qdt2m[AMPS_GPU_MAX_SPECIES];  // 0.5*q*dt/m (weight independent)
  float qw[AMPS_GPU_MAX_SPECIES];     // q*w
  float mw[AMPS_GPU_MAX_SPECIES];     // m*w
};

SpeciesTab make_species(const amps_gpu_config& c) {
  SpeciesTab t{};
  for (int s = 0; s < c.nspec; s++) {
    t.qdt2m[s] = (float)(0.5 * (c.charge[s] * c.dt / c.mass[s]));
    t.qw[s] = (float)(c.charge[s] * c.weight[s]);
    t.mw[s] = (float)(c.mass[s] * c.weight[s]);
  }
  return t;
}

// ---------------------------------------------------------------------------
// stencil packing
__global__ void k_pack_stencils(int nb, long long ncor, const int* __restrict__ nbr,
                                const double* __restrict__ Eh, const double* __restrict__ Bprev,
                                const double* __restrict__ Bcur, float* __restrict__ sp,
                                float* __restrict__ sd) {
  const int b = blockIdx.x;
  for (int s = threadIdx.x; s < AMPS_SC; s += blockDim.x) {
    int i = s % 9, j = (s / 9) % 9, k = s / 81;
    int cid = local_id(nbr, b, i, j, k);
    float4* op = reinterpret_cast<float4*>(sp + ((size_t)b * AMPS_SC + s) * AMPS_PUSH_STRIDE);
    op[0] = make_float4((float)Eh[cid], (float)Eh[ncor + cid], (float)Eh[2 * ncor + cid],
                        (float)Bprev[cid]);
    op[1] = make_float4((float)Bprev[ncor + cid], (float)Bprev[2 * ncor + cid], 0.f, 0.f);
    reinterpret_cast<float4*>(sd)[(size_t)b * AMPS_SC + s] =
        make_float4((float)Bcur[cid], (float)Bcur[ncor + cid], (float)Bcur[2 * ncor + cid], 0.f);
  }
}

// Warp-aggregated slot reservation in the destination cell: one atomic per
// distinct key in the warp, ranks inside the warp follow lane order.
__device__ __forceinline__ void reserve_slot(bool active, int key, int* __restrict__ count,
                                             int* __restrict__ rank_out, long long p) {
  unsigned act = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  unsigned peers = __match_any_sync(act, key);
  int leader = __ffs(peers) - 1;
  int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == leader) base = atomicAdd(count + key, __popc(peers));
  base = __shfl_sync(peers, base, leader);
  rank_out[p] = base + __popc(peers & lanemask_lt());
}

__device__ __forceinline__ float clamp_below8(float u) {
  return u < 8.0f ? u : 7.99999952316284180f;  // nextafterf(8, 0)
}

// ---------------------------------------------------------------------------
// Lapenta2017 push + destination key
struct PushArgs {
  const int* nbr;
  const int* start;
  const float* stencil;
  float* ux; float* uy; float* uz;
  float* vx; float* vy; float* vz;
  const uint8_t* sp;
  int* key;
  int* rank;
  int* count;
  unsigned long long* flags;
  float dtdx[3];
  float dt;
  SpeciesTab st;
};

__global__ void __launch_bounds__(256) k_push(PushArgs a) {
  extern __shared__ __align__(16) float4 s_st[];  // 729 corners x 2 float4
  __shared__ __align__(8) uint64_t bar;
  const int b = blockIdx.x;
  const int p0 = a.start[b * AMPS_CPB], p1 = a.start[(b + 1) * AMPS_CPB];
  const long long n = p1 - p0;
  const int lo = p0 + (int)(n * blockIdx.y / gridDim.y);
  const int hi = p0 + (int)(n * (blockIdx.y + 1) / gridDim.y);
  if (lo >= hi) return;
  const uint32_t bytes = AMPS_SC * AMPS_PUSH_STRIDE * sizeof(float);
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(&bar, bytes);
    bulk_copy_g2s(s_st, a.stencil + (size_t)b * AMPS_SC * AMPS_PUSH_STRIDE, bytes, &bar);
  }
  if (!mbar_wait_bounded(&bar, 0, kWaitLimit)) {
    if (threadIdx.x == 0) atomicAdd(a.flags + 2, 1ull);
    mbar_wait_bounded(&bar, 0, kWaitLimit);
    return;
  }
  unsigned long long n_out = 0, n_ulp = 0;
  for (int base = lo; base < hi; base += blockDim.x) {
    const int p = base + threadIdx.x;
    const bool act = p < hi;
    int key = 0;
    if (act) {
      float u[3] = {a.ux[p], a.uy[p], a.uz[p]};
      float v[3] = {a.vx[p], a.vy[p], a.vz[p]};
      const int s = a.sp[p];
      int ic[3];
      float f[3];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        ic[d] = min(max((int)u[d], 0), AMPS_NC - 1);
        f[d] = u[d] - (float)ic[d];
      }
      float E[3] = {0.f, 0.f, 0.f}, B[3] = {0.f, 0.f, 0.f};
#pragma unroll
      for (int cc = 0; cc < 2; cc++)
#pragma unroll
        for (int bb = 0; bb < 2; bb++)
#pragma unroll
          for (int aa = 0; aa < 2; aa++) {
            const float w = (aa ? f[0] : 1.f - f[0]) * (bb ? f[1] : 1.f - f[1]) *
                            (cc ? f[2] : 1.f - f[2]);
            const int sidx = (ic[0] + aa) + 9 * (ic[1] + bb) + 81 * (ic[2] + cc);
            const float4 q0 = s_st[2 * sidx], q1 = s_st[2 * sidx + 1];
            E[0] = fmaf(w, q0.x, E[0]);
            E[1] = fmaf(w, q0.y, E[1]);
            E[2] = fmaf(w, q0.z, E[2]);
            B[0] = fmaf(w, q0.w, B[0]);
            B[1] = fmaf(w, q1.x, B[1]);
            B[2] = fmaf(w, q1.y, B[2]);
          }
      // alpha (Eq. D.3) and v' = 2 alpha (v + qdt/2m E) - v (Eq. D.8)
      const float h = a.st.qdt2m[s];
      const float h2 = h * h;
      const float c0 = 1.0f / (1.0f + h2 * (B[0] * B[0] + B[1] * B[1] + B[2] * B[2]));
      const float P0 = -h * B[0], P1 = -h * B[1], P2 = -h * B[2];
      const float t0 = fmaf(h, E[0], v[0]), t1 = fmaf(h, E[1], v[1]), t2 = fmaf(h, E[2], v[2]);
      const float bt = h2 * (B[0] * t0 + B[1] * t1 + B[2] * t2);
      // alpha t = c0 * (t + h2 B (B.t) - P x t ... ) written out row by row
      const float a0 = c0 * (t0 + B[0] * bt + (-P2 * t1 + P1 * t2));
      const float a1 = c0 * (t1 + B[1] * bt + (P2 * t0 - P0 * t2));
      const float a2 = c0 * (t2 + B[2] * bt + (-P1 * t0 + P0 * t1));
      float vn[3] = {2.f * a0 - v[0], 2.f * a1 - v[1], 2.f * a2 - v[2]};
      int o[3];
      bool far = false, nearf = false;
#pragma unroll
      for (int d = 0; d < 3; d++) {
        float un = fmaf(vn[d], a.dtdx[d], u[d]);
        int od = (int)floorf(un * 0.125f);
        if (od > 1 || od < -1) far = true;
        od = max(-1, min(1, od));
        un -= 8.0f * (float)od;
        un = clamp_below8(fmaxf(un, 0.0f));
        o[d] = od;
        u[d] = un;
        ic[d] = min((int)un, AMPS_NC - 1);
        float fr = un - rintf(un);
        if (fabsf(fr) < 4.76837158203125e-7f) nearf = true;
      }
      if (far) n_out++;
      if (nearf) n_ulp++;
      const int nbk = (o[0] | o[1] | o[2]) ? __ldg(a.nbr + b * 27 + nbr_slot(o[0], o[1], o[2])) : b;
      key = nbk * AMPS_CPB + ic[0] + AMPS_NC * (ic[1] + AMPS_NC * ic[2]);
      a.ux[p] = u[0]; a.uy[p] = u[1]; a.uz[p] = u[2];
      a.vx[p] = vn[0]; a.vy[p] = vn[1]; a.vz[p] = vn[2];
      a.key[p] = key;
    }
    reserve_slot(act, key, a.count, a.rank, p);
  }
  if (n_out) atomicAdd(a.flags + 0, n_out);
  if (n_ulp) atomicAdd(a.flags + 1, n_ulp);
}

// ---------------------------------------------------------------------------
// exclusive scan of int counts (three passes, 1024 elements per tile)
constexpr int kScanTile = 1024;

__device__ __forceinline__ int block_excl_scan(int v, int* s_warp, int* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int nw = blockDim.x >> 5;
    int w = lane < nw ? s_warp[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < nw) s_warp[lane] = w;
  }
  __syncthreads();
  int off = wid ? s_warp[wid - 1] : 0;
  *total = s_warp[(blockDim.x >> 5) - 1];
  __syncthreads();
  return off + x - v;
}

__global__ void __launch_bounds__(256) k_scan_reduce(const int* __restrict__ in, long long n,
                                                     int* __restrict__ part) {
  __shared__ int s_warp[32];
  long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * 4;
  int s = 0;
#pragma unroll
  for (int t = 0; t < 4; t++)
    if (base + t < n) s += in[base + t];
  int total;
  block_excl_scan(s, s_warp, &total);
  if (threadIdx.x == 0) part[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_parts(int* part, int nparts) {
  __shared__ int s_warp[32];
  int carry = 0;
  for (int base = 0; base < nparts; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = i < nparts ? part[i] : 0;
    int total;
    int ex = block_excl_scan(v, s_warp, &total);
    if (i < nparts) part[i] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(256) k_scan_final(const int* __restrict__ in, long long n,
                                                    const int* __restrict__ part,
                                                    int* __restrict__ out) {
  __shared__ int s_warp[32];
  long long base = (long long)blockIdx.x * kScanTile + threadIdx.x * 4;
  int v[4], s = 0;
#pragma unroll
  for (int t = 0; t < 4; t++) {
    v[t] = (base + t < n) ? in[base + t] : 0;
    s += v[t];
  }
  int total;
  int ex = block_excl_scan(s, s_warp, &total) + part[blockIdx.x];
#pragma unroll
  for (int t = 0; t < 4; t++) {
    if (base + t < n) out[base + t] = ex;
    ex += v[t];
  }
}

// ---------------------------------------------------------------------------
struct ScatterArgs {
  const int* key; const int* rank; const int* start;
  const float* su[3]; const float* sv[3]; const uint8_t* ssp; const float* swc; const uint32_t* sid;
  float* du[3]; float* dv[3]; uint8_t* dsp; float* dwc; uint32_t* did;
  long long n;
};

__global__ void __launch_bounds__(256) k_scatter(ScatterArgs a) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < a.n;
       p += (long long)gridDim.x * blockDim.x) {
    const long long d = (long long)a.start[a.key[p]] + a.rank[p];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      a.du[c][d] = a.su[c][p];
      a.dv[c][d] = a.sv[c][p];
    }
    a.dsp[d] = a.ssp[p];
    if (a.swc) a.dwc[d] = a.swc[p];
    if (a.sid) a.did[d] = a.sid[p];
  }
}

// ---------------------------------------------------------------------------
// Deposition.  Record of one particle staged in shared memory (floats):
//   [0,36)  w_c1*w_c2 for the 36 pairs c2<=c1 (pair = c1(c1+1)/2 + c2)
//   [36,48) k*alpha in three groups of 4 (k = qW * qdt/2m / V; pad in slot 3)
//   [48,56) w_c (InterpolationCoefficientTable order)
//   [56,60) qW * alpha v (pad in slot 3)
constexpr int kRec = 60;
constexpr int kDepWarps = 8;

struct DepositArgs {
  const int* start;
  const float* stencil;
  const float* ux; const float* uy; const float* uz;
  const float* vx; const float* vy; const float* vz;
  const uint8_t* sp; const float* wc;
  float* cellM; float* cellJ;
  double* energy;
  unsigned long long* flags;
  float inv_vol;
  SpeciesTab st;
};

__global__ void __launch_bounds__(256) k_deposit(DepositArgs a) {
  extern __shared__ __align__(16) float4 s_dyn[];
  float4* s_B = s_dyn;                                  // 729 float4
  float* s_rec = reinterpret_cast<float*>(s_dyn + AMPS_SC);  // kDepWarps * 32 * kRec
  __shared__ __align__(8) uint64_t bar;
  __shared__ double s_en[kDepWarps];
  const int b = blockIdx.x, k = blockIdx.y;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t bytes = AMPS_SC * AMPS_DEP_STRIDE * sizeof(float);
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    mbar_arrive_expect_tx(&bar, bytes);
    bulk_copy_g2s(s_B, a.stencil + (size_t)b * AMPS_SC * AMPS_DEP_STRIDE, bytes, &bar);
  }
  if (!mbar_wait_bounded(&bar, 0, kWaitLimit)) {
    if (threadIdx.x == 0) atomicAdd(a.flags + 2, 1ull);
    mbar_wait_bounded(&bar, 0, kWaitLimit);
    return;
  }
  float* rec = s_rec + wid * 32 * kRec;
  double en = 0.0;
  const int j = wid;
  // lane roles in the accumulation phase
  const bool tile = lane < 29;
  const int offA = lane < 27 ? 4 * (lane / 3) : 48 + 4 * (lane - 27);
  const int offB = lane < 27 ? 36 + 4 * (lane % 3) : 56;
  for (int i = 0; i < AMPS_NC; i++) {
    const int cl = i + AMPS_NC * (j + AMPS_NC * k);
    const long long cid = (long long)b * AMPS_CPB + cl;
    const int p0 = a.start[cid], p1 = a.start[cid + 1];
    float sum[12], cmp[12];
#pragma unroll
    for (int e = 0; e < 12; e++) { sum[e] = 0.f; cmp[e] = 0.f; }
    for (int base = p0; base < p1; base += 32) {
      const int p = base + lane;
      if (p < p1) {
        const float u0 = a.ux[p], u1 = a.uy[p], u2 = a.uz[p];
        const float v0 = a.vx[p], v1 = a.vy[p], v2 = a.vz[p];
        const int s = a.sp[p];
        const float wcorr = a.wc ? a.wc[p] : 1.0f;
        const float fx = fminf(fmaxf(u0 - (float)i, 0.f), 1.f);
        const float fy = fminf(fmaxf(u1 - (float)j, 0.f), 1.f);
        const float fz = fminf(fmaxf(u2 - (float)k, 0.f), 1.f);
        const float gx = 1.f - fx, gy = 1.f - fy, gz = 1.f - fz;
        float w[8];
        w[0] = gx * gy * gz; w[1] = fx * gy * gz; w[2] = fx * fy * gz; w[3] = gx * fy * gz;
        w[4] = gx * gy * fz; w[5] = fx * gy * fz; w[6] = fx * fy * fz; w[7] = gx * fy * fz;
        const int sb = i + 9 * (j + 9 * k);
        const int coff[8] = {0, 1, 10, 9, 81, 82, 91, 90};
        float B0 = 0.f, B1 = 0.f, B2 = 0.f;
#pragma unroll
        for (int c = 0; c < 8; c++) {
          const float4 q = s_B[sb + coff[c]];
          B0 = fmaf(w[c], q.x, B0);
          B1 = fmaf(w[c], q.y, B1);
          B2 = fmaf(w[c], q.z, B2);
        }
        const float h = a.st.qdt2m[s];
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
        const float qW = a.st.qw[s] * wcorr;
        const float mW = a.st.mw[s] * wcorr;
        const float kc = qW * h * a.inv_vol;
        en += 0.5 * (double)mW * ((double)v0 * v0 + (double)v1 * v1 + (double)v2 * v2);
        float* r = rec + lane * kRec;
        float4* r4 = reinterpret_cast<float4*>(r);
        float ww[36];
        {
          int pr = 0;
#pragma unroll
          for (int c1 = 0; c1 < 8; c1++)
#pragma unroll
            for (int c2 = 0; c2 <= c1; c2++, pr++) ww[pr] = w[c1] * w[c2];
        }
#pragma unroll
        for (int t = 0; t < 9; t++) r4[t] = make_float4(ww[4 * t], ww[4 * t + 1], ww[4 * t + 2], ww[4 * t + 3]);
        r4[9] = make_float4(kc * al[0], kc * al[1], kc * al[2], 0.f);
        r4[10] = make_float4(kc * al[3], kc * al[4], kc * al[5], 0.f);
        r4[11] = make_float4(kc * al[6], kc * al[7], kc * al[8], 0.f);
        r4[12] = make_float4(w[0], w[1], w[2], w[3]);
        r4[13] = make_float4(w[4], w[5], w[6], w[7]);
        const float vr0 = al[0] * v0 + al[1] * v1 + al[2] * v2;
        const float vr1 = al[3] * v0 + al[4] * v1 + al[5] * v2;
        const float vr2 = al[6] * v0 + al[7] * v1 + al[8] * v2;
        r4[14] = make_float4(qW * vr0, qW * vr1, qW * vr2, 0.f);
      }
      __syncwarp();
      const int cnt = min(32, p1 - base);
      if (tile) {
        float acc[12];
#pragma unroll
        for (int e = 0; e < 12; e++) acc[e] = 0.f;
        for (int r = 0; r < cnt; r++) {
          const float4 A = *reinterpret_cast<const float4*>(rec + r * kRec + offA);
          const float4 Bv = *reinterpret_cast<const float4*>(rec + r * kRec + offB);
          const float av[4] = {A.x, A.y, A.z, A.w};
#pragma unroll
          for (int q = 0; q < 4; q++) {
            acc[3 * q + 0] = fmaf(av[q], Bv.x, acc[3 * q + 0]);
            acc[3 * q + 1] = fmaf(av[q], Bv.y, acc[3 * q + 1]);
            acc[3 * q + 2] = fmaf(av[q], Bv.z, acc[3 * q + 2]);
          }
        }
        // compensated (Kahan) add of the chunk sum
#pragma unroll
        for (int e = 0; e < 12; e++) {
          const float y = acc[e] - cmp[e];
          const float t = sum[e] + y;
          cmp[e] = (t - sum[e]) - y;
          sum[e] = t;
        }
      }
      __syncwarp();
    }
    // flush the cell partials
    if (lane < 27) {
      const int g = lane / 3, hh = lane % 3;
      float* dst = a.cellM + cid * 324;
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int e = 0; e < 3; e++) dst[(4 * g + q) * 9 + 3 * hh + e] = sum[3 * q + e] - cmp[3 * q + e];
    } else if (lane < 29) {
      const int g = lane - 27;
      float* dst = a.cellJ + cid * 24;
#pragma unroll
      for (int q = 0; q < 4; q++)
#pragma unroll
        for (int e = 0; e < 3; e++) dst[(4 * g + q) * 3 + e] = sum[3 * q + e] - cmp[3 * q + e];
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) en += __shfl_xor_sync(0xffffffffu, en, o);
  if (lane == 0) s_en[wid] = en;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kDepWarps; w++) t += s_en[w];
    atomicAdd(a.energy, t);
  }
}

// ---------------------------------------------------------------------------
// Corner assembly.  For corner c and each of its 8 cells, the pair (c, c2) of
// that cell lands in slot(c2 - c) of M_c.  The 64 (slot, cell, pair) entries are
// grouped by slot so each output slot is written once.
struct AsmEntry {
  unsigned char slot, cell, pair, pad;
};
__constant__ AsmEntry c_asm[64];
__constant__ unsigned char c_asm_corner[8];  // table index of the corner inside cell co

__global__ void __launch_bounds__(256) k_assemble(long long ncor, const int* __restrict__ nbr,
                                                  const float* __restrict__ cellM,
                                                  const float* __restrict__ cellJ, double inv_vol,
                                                  double* __restrict__ M, double* __restrict__ J) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncor) return;
  const int b = (int)(c / AMPS_CPB), l = (int)(c % AMPS_CPB);
  const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
  int cell[8];
#pragma unroll
  for (int co = 0; co < 8; co++)
    cell[co] = local_id(nbr, b, i - (co & 1), j - ((co >> 1) & 1), k - ((co >> 2) & 1));
  double acc[9];
  int cur = c_asm[0].slot;
#pragma unroll
  for (int e = 0; e < 9; e++) acc[e] = 0.0;
  for (int t = 0; t < 64; t++) {
    const AsmEntry en = c_asm[t];
    if (en.slot != cur) {
#pragma unroll
      for (int e = 0; e < 9; e++) {
        M[(size_t)(cur * 9 + e) * ncor + c] = acc[e];
        acc[e] = 0.0;
      }
      cur = en.slot;
    }
    const float* src = cellM + (size_t)cell[en.cell] * 324 + en.pair * 9;
#pragma unroll
    for (int e = 0; e < 9; e++) acc[e] += (double)src[e];
  }
#pragma unroll
  for (int e = 0; e < 9; e++) M[(size_t)(cur * 9 + e) * ncor + c] = acc[e];
  double jj[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int co = 0; co < 8; co++) {
    const float* src = cellJ + (size_t)cell[co] * 24 + c_asm_corner[co] * 3;
    jj[0] += (double)src[0];
    jj[1] += (double)src[1];
    jj[2] += (double)src[2];
  }
  J[c] = jj[0] * inv_vol;
  J[ncor + c] = jj[1] * inv_vol;
  J[2 * ncor + c] = jj[2] * inv_vol;
}

// ---------------------------------------------------------------------------
// Import: FP64 physical position -> block, cell, FP32 offset (findTreeNode +
// FindCellIndex + periodic exchange rules), then the same slot reservation.
struct ImportArgs {
  const double* x; const double* v; const uint8_t* sp; const double* wc;
  float* ux; float* uy; float* uz; float* vx; float* vy; float* vz;
  uint8_t* dsp; float* dwc; uint32_t* did;
  int* key; int* rank; int* count;
  unsigned long long* flags;
  long long n;
  int nbk[3];
  double x0[3], dx[3];
  int nspec;
};

__global__ void __launch_bounds__(256) k_import(ImportArgs a) {
  for (long long base = (long long)blockIdx.x * blockDim.x; base < a.n;
       base += (long long)gridDim.x * blockDim.x) {
    const long long p = base + threadIdx.x;
    const bool act = p < a.n;
    int key = 0;
    if (act) {
      int bx[3], ic[3];
      float uf[3];
      for (int d = 0; d < 3; d++) {
        double x = a.x[3 * p + d];
        const double L = AMPS_NC * a.dx[d];
        int bb = (int)floor((x - a.x0[d]) / L);
        double xmin = a.x0[d] + bb * L;
        if (x < xmin) { bb--; xmin = a.x0[d] + bb * L; }
        if (x >= xmin + L) { bb++; xmin = a.x0[d] + bb * L; }
        int ci = (int)((x - xmin) / a.dx[d]);
        if (ci >= AMPS_NC) ci = AMPS_NC - 1;
        if (ci < 0) ci = 0;
        if (bb < 0 || bb >= a.nbk[d]) {
          int br = ((bb % a.nbk[d]) + a.nbk[d]) % a.nbk[d];
          double xr = a.x0[d] + br * L;
          x += xr - xmin;
          if (x < xr) x = xr;
          if (x >= xr + L) x = (xr + L) - 1.0E-10 * L;
          bb = br;
          xmin = xr;
          if (bb < 0 || bb >= a.nbk[d]) atomicAdd(a.flags + 2, 1ull);
        }
        float u = (float)((x - xmin) / a.dx[d]);
        // keep the FP32 offset inside the FP64 cell
        if (u < (float)ci) u = (float)ci;
        if (u >= (float)(ci + 1)) u = nextafterf((float)(ci + 1), 0.0f);
        uf[d] = u;
        bx[d] = bb;
        ic[d] = ci;
      }
      const int blk = bx[0] + a.nbk[0] * (bx[1] + a.nbk[1] * bx[2]);
      key = blk * AMPS_CPB + ic[0] + AMPS_NC * (ic[1] + AMPS_NC * ic[2]);
      a.ux[p] = uf[0]; a.uy[p] = uf[1]; a.uz[p] = uf[2];
      a.vx[p] = (float)a.v[3 * p]; a.vy[p] = (float)a.v[3 * p + 1]; a.vz[p] = (float)a.v[3 * p + 2];
      int s = a.sp[p];
      if (s >= a.nspec) atomicAdd(a.flags + 2, 1ull);
      a.dsp[p] = (uint8_t)s;
      if (a.dwc) a.dwc[p] = a.wc ? (float)a.wc[p] : 1.0f;
      if (a.did) a.did[p] = (uint32_t)p;
      a.key[p] = key;
    }
    reserve_slot(act, key, a.count, a.rank, p);
  }
}

// Local import: block id + FP32 offsets already given.
__global__ void __launch_bounds__(256) k_import_local(long long n, const int* __restrict__ blk,
                                                      float* ux, float* uy, float* uz,
                                                      uint32_t* did, int* key, int* rank,
                                                      int* count, int nb,
                                                      unsigned long long* flags) {
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n;
       base += (long long)gridDim.x * blockDim.x) {
    const long long p = base + threadIdx.x;
    const bool act = p < n;
    int kk = 0;
    if (act) {
      float u[3] = {ux[p], uy[p], uz[p]};
      int ic[3];
      for (int d = 0; d < 3; d++) {
        if (!(u[d] >= 0.f && u[d] < 8.f)) atomicAdd(flags + 2, 1ull);
        u[d] = clamp_below8(fmaxf(u[d], 0.f));
        ic[d] = min((int)u[d], AMPS_NC - 1);
      }
      ux[p] = u[0]; uy[p] = u[1]; uz[p] = u[2];
      int b = blk[p];
      if (b < 0 || b >= nb) { atomicAdd(flags + 2, 1ull); b = 0; }
      kk = b * AMPS_CPB + ic[0] + AMPS_NC * (ic[1] + AMPS_NC * ic[2]);
      key[p] = kk;
      if (did) did[p] = (uint32_t)p;
    }
    reserve_slot(act, kk, count, rank, p);
  }
}

int grid_for(long long n, int threads) {
  long long g = (n + threads - 1) / threads;
  if (g > 152LL * 64) g = 152LL * 64;
  if (g < 1) g = 1;
  return (int)g;
}

bool g_asm_ready = false;

void init_asm_table() {
  if (g_asm_ready) return;
  static const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  auto tidx = [&](int x, int y, int z) {
    for (int t = 0; t < 8; t++)
      if (off[t][0] == x && off[t][1] == y && off[t][2] == z) return t;
    return -1;
  };
  AsmEntry e[64];
  unsigned char corner_of[8];
  int n = 0;
  for (int slot = 0; slot < 27; slot++)
    for (int co = 0; co < 8; co++) {
      // cell = corner + (-(co&1), -((co>>1)&1), -((co>>2)&1)); the corner sits at
      // local offset ((co&1), (co>>1)&1, (co>>2)&1) inside that cell
      int lx = co & 1, ly = (co >> 1) & 1, lz = (co >> 2) & 1;
      int c1 = tidx(lx, ly, lz);
      corner_of[co] = (unsigned char)c1;
      for (int c2 = 0; c2 < 8; c2++) {
        int dx = off[c2][0] - lx, dy = off[c2][1] - ly, dz = off[c2][2] - lz;
        if (mm_slot(dx, dy, dz) != slot) continue;
        int hi = c1 > c2 ? c1 : c2, lo = c1 > c2 ? c2 : c1;
        e[n].slot = (unsigned char)slot;
        e[n].cell = (unsigned char)co;
        e[n].pair = (unsigned char)(hi * (hi + 1) / 2 + lo);
        e[n].pad = 0;
        n++;
      }
    }
  cudaMemcpyToSymbol(c_asm, e, sizeof(e));
  cudaMemcpyToSymbol(c_asm_corner, corner_of, sizeof(corner_of));
  g_asm_ready = true;
}

}  // namespace

// ===========================================================================
// launchers
cudaError_t launch_pack_stencils(amps_gpu_ctx* c, const double* Eh, const double* Bprev,
                                 const double* Bcur) {
  TimedLaunch t(c, "pack_stencils");
  k_pack_stencils<<<c->nb, 256, 0, c->stream>>>(c->nb, c->ncor, c->d_nbr, Eh, Bprev, Bcur,
                                                 c->d_stencil_push, c->d_stencil_dep);
  return cudaGetLastError();
}

static int push_splits(const amps_gpu_ctx* c) {
  long long per = c->np / (c->nb > 0 ? c->nb : 1);
  long long s = per / 4096;
  if (s < 1) s = 1;
  if (s > 256) s = 256;
  return (int)s;
}

cudaError_t launch_push(amps_gpu_ctx* c) {
  const int cur = c->cur;
  cudaError_t e = cudaMemsetAsync(c->d_count, 0, sizeof(int) * (c->ncor + 1), c->stream);
  if (e != cudaSuccess) return e;
  PushArgs a;
  a.nbr = c->d_nbr;
  a.start = c->d_start;
  a.stencil = c->d_stencil_push;
  a.ux = c->d_u[cur][0]; a.uy = c->d_u[cur][1]; a.uz = c->d_u[cur][2];
  a.vx = c->d_v[cur][0]; a.vy = c->d_v[cur][1]; a.vz = c->d_v[cur][2];
  a.sp = c->d_sp[cur];
  a.key = c->d_key; a.rank = c->d_rank; a.count = c->d_count;
  a.flags = c->d_flags;
  for (int d = 0; d < 3; d++) a.dtdx[d] = (float)(c->cfg.dt / c->cfg.dx[d]);
  a.dt = (float)c->cfg.dt;
  a.st = make_species(c->cfg);
  const size_t smem = AMPS_SC * AMPS_PUSH_STRIDE * sizeof(float);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_push, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  TimedLaunch t(c, "push");
  dim3 grid(c->nb, push_splits(c));
  k_push<<<grid, 256, smem, c->stream>>>(a);
  return cudaGetLastError();
}

static cudaError_t scan_counts(amps_gpu_ctx* c) {
  const long long n = c->ncor + 1;
  const int tiles = (int)((n + kScanTile - 1) / kScanTile);
  TimedLaunch t(c, "scan", 3);
  k_scan_reduce<<<tiles, 256, 0, c->stream>>>(c->d_count, n, c->d_scan_part);
  k_scan_parts<<<1, 1024, 0, c->stream>>>(c->d_scan_part, tiles);
  k_scan_final<<<tiles, 256, 0, c->stream>>>(c->d_count, n, c->d_scan_part, c->d_start);
  return cudaGetLastError();
}

cudaError_t launch_rebin(amps_gpu_ctx* c) {
  cudaError_t e = scan_counts(c);
  if (e != cudaSuccess) return e;
  const int s = c->cur, d = s ^ 1;
  ScatterArgs a;
  a.key = c->d_key; a.rank = c->d_rank; a.start = c->d_start;
  for (int q = 0; q < 3; q++) {
    a.su[q] = c->d_u[s][q]; a.sv[q] = c->d_v[s][q];
    a.du[q] = c->d_u[d][q]; a.dv[q] = c->d_v[d][q];
  }
  a.ssp = c->d_sp[s]; a.dsp = c->d_sp[d];
  a.swc = c->has_wcorr ? c->d_wc[s] : nullptr;
  a.dwc = c->has_wcorr ? c->d_wc[d] : nullptr;
  a.sid = c->cfg.track_ids ? c->d_id[s] : nullptr;
  a.did = c->cfg.track_ids ? c->d_id[d] : nullptr;
  a.n = c->np;
  {
    TimedLaunch t(c, "scatter");
    k_scatter<<<grid_for(c->np, 256), 256, 0, c->stream>>>(a);
  }
  c->cur = d;
  return cudaGetLastError();
}

cudaError_t launch_deposit(amps_gpu_ctx* c) {
  init_asm_table();
  const int cur = c->cur;
  DepositArgs a;
  a.start = c->d_start;
  a.stencil = c->d_stencil_dep;
  a.ux = c->d_u[cur][0]; a.uy = c->d_u[cur][1]; a.uz = c->d_u[cur][2];
  a.vx = c->d_v[cur][0]; a.vy = c->d_v[cur][1]; a.vz = c->d_v[cur][2];
  a.sp = c->d_sp[cur];
  a.wc = c->has_wcorr ? c->d_wc[cur] : nullptr;
  a.cellM = c->d_cellM; a.cellJ = c->d_cellJ;
  a.energy = c->d_energy;
  a.flags = c->d_flags;
  a.inv_vol = (float)(1.0 / (c->cfg.dx[0] * c->cfg.dx[1] * c->cfg.dx[2]));
  a.st = make_species(c->cfg);
  const size_t smem = AMPS_SC * sizeof(float4) + kDepWarps * 32 * kRec * sizeof(float);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  cudaError_t e = cudaMemsetAsync(c->d_energy, 0, sizeof(double), c->stream);
  if (e != cudaSuccess) return e;
  {
    TimedLaunch t(c, "deposit");
    k_deposit<<<dim3(c->nb, AMPS_NC), kDepWarps * 32, smem, c->stream>>>(a);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  {
    TimedLaunch t(c, "assemble");
    const double inv_vol = 1.0 / (c->cfg.dx[0] * c->cfg.dx[1] * c->cfg.dx[2]);
    k_assemble<<<(unsigned)((c->ncor + 255) / 256), 256, 0, c->stream>>>(
        c->ncor, c->d_nbr, c->d_cellM, c->d_cellJ, inv_vol, c->d_M, c->d_J);
  }
  return cudaGetLastError();
}

// Import helpers used by the C ABI (capi.cu)
cudaError_t launch_import_fp64(amps_gpu_ctx* c, const double* d_x, const double* d_v,
                               const uint8_t* d_spec_in, const double* d_wc, long long n) {
  cudaError_t e = cudaMemsetAsync(c->d_count, 0, sizeof(int) * (c->ncor + 1), c->stream);
  if (e != cudaSuccess) return e;
  const int cur = c->cur;
  ImportArgs a;
  a.x = d_x; a.v = d_v; a.sp = d_spec_in; a.wc = d_wc;
  a.ux = c->d_u[cur][0]; a.uy = c->d_u[cur][1]; a.uz = c->d_u[cur][2];
  a.vx = c->d_v[cur][0]; a.vy = c->d_v[cur][1]; a.vz = c->d_v[cur][2];
  a.dsp = c->d_sp[cur];
  a.dwc = c->has_wcorr ? c->d_wc[cur] : nullptr;
  a.did = c->cfg.track_ids ? c->d_id[cur] : nullptr;
  a.key = c->d_key; a.rank = c->d_rank; a.count = c->d_count;
  a.flags = c->d_flags;
  a.n = n;
  a.nbk[0] = c->cfg.nbx; a.nbk[1] = c->cfg.nby; a.nbk[2] = c->cfg.nbz;
  for (int d = 0; d < 3; d++) { a.x0[d] = c->cfg.x0[d]; a.dx[d] = c->cfg.dx[d]; }
  a.nspec = c->cfg.nspec;
  {
    TimedLaunch t(c, "import");
    k_import<<<grid_for(n, 256), 256, 0, c->stream>>>(a);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  c->np = n;
  return launch_rebin(c);
}

cudaError_t launch_import_local(amps_gpu_ctx* c, const int32_t* d_block, long long n) {
  cudaError_t e = cudaMemsetAsync(c->d_count, 0, sizeof(int) * (c->ncor + 1), c->stream);
  if (e != cudaSuccess) return e;
  const int cur = c->cur;
  {
    TimedLaunch t(c, "import");
    k_import_local<<<grid_for(n, 256), 256, 0, c->stream>>>(
        n, d_block, c->d_u[cur][0], c->d_u[cur][1], c->d_u[cur][2],
        c->cfg.track_ids ? c->d_id[cur] : nullptr, c->d_key, c->d_rank, c->d_count, c->nb,
        c->d_flags);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  c->np = n;
  return launch_rebin(c);
}

// Export: physical FP64 positions, velocities, block and cell per particle in
// device order.
__global__ void __launch_bounds__(256) k_export(long long ncells, const int* __restrict__ start,
                                                const float* ux, const float* uy, const float* uz,
                                                const float* vx, const float* vy, const float* vz,
                                                int nbx, int nby, double x00, double x01,
                                                double x02, double dx0, double dx1, double dx2,
                                                double* x, double* v, int32_t* blk, int32_t* cel) {
  const long long cid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cid >= ncells) return;
  const int b = (int)(cid / AMPS_CPB), l = (int)(cid % AMPS_CPB);
  const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
  const double o0 = x00 + bx * (AMPS_NC * dx0), o1 = x01 + by * (AMPS_NC * dx1),
               o2 = x02 + bz * (AMPS_NC * dx2);
  for (int p = start[cid]; p < start[cid + 1]; p++) {
    if (x) {
      x[3LL * p] = o0 + (double)ux[p] * dx0;
      x[3LL * p + 1] = o1 + (double)uy[p] * dx1;
      x[3LL * p + 2] = o2 + (double)uz[p] * dx2;
    }
    if (v) {
      v[3LL * p] = vx[p];
      v[3LL * p + 1] = vy[p];
      v[3LL * p + 2] = vz[p];
    }
    if (blk) blk[p] = b;
    if (cel) cel[p] = l;
  }
}

cudaError_t launch_export(amps_gpu_ctx* c, double* d_x, double* d_v, int32_t* d_blk,
                          int32_t* d_cel) {
  const int cur = c->cur;
  TimedLaunch t(c, "export");
  k_export<<<(unsigned)((c->ncor + 255) / 256), 256, 0, c->stream>>>(
      c->ncor, c->d_start, c->d_u[cur][0], c->d_u[cur][1], c->d_u[cur][2], c->d_v[cur][0],
      c->d_v[cur][1], c->d_v[cur][2], c->cfg.nbx, c->cfg.nby, c->cfg.x0[0], c->cfg.x0[1],
      c->cfg.x0[2], c->cfg.dx[0], c->cfg.dx[1], c->cfg.dx[2], d_x, d_v, d_blk, d_cel);
  return cudaGetLastError();
}
