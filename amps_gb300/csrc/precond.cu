// Learned right preconditioner for the ECSIM field solve: a block-local
// convolutional network trained on residual/correction pairs that the Jacobi
// GMRES solves themselves produce.  No reference counterpart (the reference's
// GMRES takes PrecondParam 0/1, pic_field_solver_ecsim.cpp:6232).
//
// Per mesh block the network sees x = D r (the Jacobi-scaled residual) on the
// block's 8^3 owned corners plus a 1-corner halo (a 10^3 region R), applies
// three 3x3x3 convolutions 3 -> 32 -> 32 -> 3 with zero padding at the edge of
// R and no activation, and returns y on the owned corners: z = x + y.  Being
// linear and bias-free, P r = D r + N(D r) is a fixed linear operator (up to
// the rounding of its FP32/BF16 arithmetic, which the flexible GMRES absorbs).
//
// Layouts: activations [sample][voxel of R, (k*10 + j)*10 + i][channel];
// weights [tap (dx+1)+3(dy+1)+9(dz+1)][in channel][out channel].
//
// Kernels here (FP32 CUDA cores): k_conv (forward; with flipped, transposed
// weights also the input gradient), k_wgrad (weight gradient), k_loss, k_adam,
// k_harvest (pairs from a solve), k_gather_region / k_scatter_z (inference on
// the mesh).  The BF16 tensor-core inference kernel is in precond_tc.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <random>
#include <vector>

#include "common.cuh"
#include "precond.cuh"

namespace {

constexpr int kR = 10;            // region edge
constexpr int kRV = kR * kR * kR;  // region voxels
constexpr int kOwn = 512;

__host__ __device__ __forceinline__ int tap_dx(int t) { return t % 3 - 1; }
__host__ __device__ __forceinline__ int tap_dy(int t) { return (t / 3) % 3 - 1; }
__host__ __device__ __forceinline__ int tap_dz(int t) { return t / 9 - 1; }
__device__ __forceinline__ bool owned_voxel(int i, int j, int k) {
  return i >= 1 && i <= 8 && j >= 1 && j <= 8 && k >= 1 && k <= 8;
}

// out[s][v][o] = sum_t sum_c W[t][c][o] in[s][v + off_t][c]   (zero outside R)
// grid (10 planes, S), 256 threads; one plane of R per CTA.
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_conv(const float* __restrict__ in,
                                              const float* __restrict__ W,
                                              float* __restrict__ out, int owned_only) {
  constexpr int CP = CIN + 1;  // padded smem row (bank spread)
  extern __shared__ float smem[];
  float* sW = smem;                         // 27*CIN*COUT
  float* sIn = smem + 27 * CIN * COUT;      // 3 planes x 100 voxels x CP
  const int kz = blockIdx.x, s = blockIdx.y;
  for (int t = threadIdx.x; t < 27 * CIN * COUT; t += blockDim.x) sW[t] = W[t];
  const float* ins = in + (size_t)s * kRV * CIN;
  for (int t = threadIdx.x; t < 300 * CIN; t += blockDim.x) {
    const int c = t % CIN, pv = t / CIN, pl = pv / 100, v = pv % 100;
    const int z = kz + pl - 1;
    sIn[pv * CP + c] = (z >= 0 && z < kR) ? ins[(size_t)(z * 100 + v) * CIN + c] : 0.f;
  }
  __syncthreads();
  constexpr int OG = COUT >= 8 ? 8 : COUT;  // output channels per thread
  constexpr int NG = COUT / OG;
  float* outs = out + (size_t)s * kRV * COUT;
  for (int item = threadIdx.x; item < 100 * NG; item += blockDim.x) {
    const int v = item % 100, og = item / 100;
    const int i = v % 10, j = v / 10;
    float acc[OG];
#pragma unroll
    for (int o = 0; o < OG; o++) acc[o] = 0.f;
    const bool active = !owned_only || owned_voxel(i, j, kz);
    if (active) {
      for (int t = 0; t < 27; t++) {
        const int ii = i + tap_dx(t), jj = j + tap_dy(t), pl = 1 + tap_dz(t);
        if (ii < 0 || ii >= kR || jj < 0 || jj >= kR) continue;
        const float* src = sIn + (pl * 100 + jj * 10 + ii) * CP;
        const float* w = sW + t * CIN * COUT + og * OG;
#pragma unroll 4
        for (int c = 0; c < CIN; c++) {
          const float a = src[c];
#pragma unroll
          for (int o = 0; o < OG; o++) acc[o] = fmaf(a, w[c * COUT + o], acc[o]);
        }
      }
    }
#pragma unroll
    for (int o = 0; o < OG; o++) outs[(size_t)(kz * 100 + v) * COUT + og * OG + o] = acc[o];
  }
}

// Wt[t][o][c] = W[26 - t][c][o]: the input gradient is a convolution of the
// output gradient with flipped taps and transposed channels
__global__ void k_flip(const float* __restrict__ W, float* __restrict__ Wt, int cin, int cout) {
  const int n = 27 * cin * cout;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int t = q / (cin * cout), r = q % (cin * cout), c = r / cout, o = r % cout;
    Wt[((size_t)(26 - t) * cout + o) * cin + c] = W[q];
  }
}

// dW[t][c][o] += sum_{s,v} dout[s][v][o] in[s][v + off_t][c]
// grid (27 taps, sample chunks), 256 threads; voxel tiles of 64 in shared memory.
template <int CIN, int COUT>
__global__ void __launch_bounds__(256) k_wgrad(int S, int chunk, const float* __restrict__ dout,
                                               const float* __restrict__ in,
                                               float* __restrict__ dW) {
  constexpr int TV = 64;
  constexpr int NP = CIN * COUT;
  constexpr int PT = (NP + 255) / 256;  // (c,o) pairs per thread
  __shared__ float sD[TV][COUT + 1];
  __shared__ float sI[TV][CIN + 1];
  const int t = blockIdx.x;
  const int dx = tap_dx(t), dy = tap_dy(t), dz = tap_dz(t);
  const int s0 = blockIdx.y * chunk, s1 = min(S, s0 + chunk);
  float acc[PT];
#pragma unroll
  for (int q = 0; q < PT; q++) acc[q] = 0.f;
  for (int s = s0; s < s1; s++) {
    const float* ds = dout + (size_t)s * kRV * COUT;
    const float* is = in + (size_t)s * kRV * CIN;
    for (int v0 = 0; v0 < kRV; v0 += TV) {
      __syncthreads();
      for (int q = threadIdx.x; q < TV * COUT; q += blockDim.x) {
        const int vv = q / COUT, o = q % COUT, v = v0 + vv;
        sD[vv][o] = v < kRV ? ds[(size_t)v * COUT + o] : 0.f;
      }
      for (int q = threadIdx.x; q < TV * CIN; q += blockDim.x) {
        const int vv = q / CIN, c = q % CIN, v = v0 + vv;
        float a = 0.f;
        if (v < kRV) {
          const int i = v % 10 + dx, j = (v / 10) % 10 + dy, k = v / 100 + dz;
          if (i >= 0 && i < kR && j >= 0 && j < kR && k >= 0 && k < kR)
            a = is[(size_t)((k * 10 + j) * 10 + i) * CIN + c];
        }
        sI[vv][c] = a;
      }
      __syncthreads();
#pragma unroll
      for (int q = 0; q < PT; q++) {
        const int pidx = threadIdx.x + q * 256;
        if (pidx < NP) {
          const int c = pidx / COUT, o = pidx % COUT;
          float a = acc[q];
#pragma unroll 8
          for (int vv = 0; vv < TV; vv++) a = fmaf(sD[vv][o], sI[vv][c], a);
          acc[q] = a;
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < PT; q++) {
    const int pidx = threadIdx.x + q * 256;
    if (pidx < NP) atomicAdd(dW + (size_t)t * NP + pidx, acc[q]);
  }
}

// loss = mean over owned voxels, channels of (x + y - e)^2; dy = dloss/dy
__global__ void __launch_bounds__(256) k_loss(int S, const float* __restrict__ x,
                                              const float* __restrict__ y,
                                              const float* __restrict__ e,
                                              float* __restrict__ dy, double* __restrict__ loss) {
  const long long n = (long long)S * kRV;
  const float scale = 1.0f / (float)((double)S * kOwn * 3);
  double acc = 0.0;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int s = (int)(q / kRV), v = (int)(q % kRV);
    const int i = v % 10, j = (v / 10) % 10, k = v / 100;
    if (owned_voxel(i, j, k)) {
      const int o = (k - 1) * 64 + (j - 1) * 8 + (i - 1);
#pragma unroll
      for (int ch = 0; ch < 3; ch++) {
        const float r = x[q * 3 + ch] + y[q * 3 + ch] - e[((size_t)s * kOwn + o) * 3 + ch];
        acc += (double)r * r;
        dy[q * 3 + ch] = 2.0f * r * scale;
      }
    } else {
#pragma unroll
      for (int ch = 0; ch < 3; ch++) dy[q * 3 + ch] = 0.f;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  __shared__ double sh[8];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    atomicAdd(loss, t * (double)scale);
  }
}

__global__ void k_adam(int n, float* __restrict__ w, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                       float c1, float c2, float eps) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const float gg = g[q];
    const float mm = b1 * m[q] + (1.f - b1) * gg;
    const float vv = b2 * v[q] + (1.f - b2) * gg * gg;
    m[q] = mm;
    v[q] = vv;
    w[q] -= lr * (mm * c1) / (sqrtf(vv * c2) + eps);
  }
}

// samples perm[first..first+S) -> contiguous work buffers
__global__ void k_gather_batch(int S, const int* __restrict__ perm, long long first,
                               const float* __restrict__ sx, const float* __restrict__ se,
                               float* __restrict__ wx, float* __restrict__ we) {
  const int s = blockIdx.x;
  const long long src = perm[first + s];
  for (int q = threadIdx.x; q < kRV * 3; q += blockDim.x)
    wx[(size_t)s * kRV * 3 + q] = sx[src * kRV * 3 + q];
  for (int q = threadIdx.x; q < kOwn * 3; q += blockDim.x)
    we[(size_t)s * kOwn * 3 + q] = se[src * kOwn * 3 + q];
}

// One block per mesh block: x = dinv .* r on R (FP32, zero where the region
// map has no corner) and e on the corners the block writes (optionally scaled
// by dinv; where it writes none, e = x so that the target correction is 0),
// both divided by the RMS of x over R.
__global__ void __launch_bounds__(256) k_harvest(int nb, long long nvc, const int* __restrict__ in_map,
                                                 const int* __restrict__ hs, const int* __restrict__ hp,
                                                 const double* __restrict__ hw,
                                                 const int* __restrict__ out_map,
                                                 const double* __restrict__ r,
                                                 const double* __restrict__ e,
                                                 const double* __restrict__ dinv, int e_scaled,
                                                 float* __restrict__ sx, float* __restrict__ se,
                                                 long long slot0, long long cap) {
  const int b = blockIdx.x;
  const long long s = slot0 + b;
  if (s >= cap) return;
  __shared__ float sxv[kRV * 3];
  __shared__ double sh[8];
  double ss = 0.0;
  for (int q = threadIdx.x; q < kRV; q += blockDim.x) {
    const int id = in_map[(size_t)b * kRV + q];
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {
      const double v = pc_input(id, ch, nvc, r, dinv, hs, hp, hw);
      sxv[q * 3 + ch] = (float)v;
      ss += v * v;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = ss;
  __syncthreads();
  double tot = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += sh[w];
  const double rms = sqrt(tot / (kRV * 3));
  const float inv = rms > 0.0 ? (float)(1.0 / rms) : 0.f;
  for (int q = threadIdx.x; q < kRV * 3; q += blockDim.x) sx[s * kRV * 3 + q] = sxv[q] * inv;
  for (int q = threadIdx.x; q < kOwn; q += blockDim.x) {
    const int id = out_map[(size_t)b * kOwn + q];  // corner q = i + 8j + 64k of the block
    const int vox = (((q >> 6) + 1) * 10 + ((q >> 3) & 7) + 1) * 10 + (q & 7) + 1;
#pragma unroll
    for (int ch = 0; ch < 3; ch++) {
      float t;
      if (id >= 0) {
        double v = e[ch * nvc + id];
        if (e_scaled) v *= dinv[ch * nvc + id];
        t = (float)(v * (rms > 0.0 ? 1.0 / rms : 0.0));
      } else {
        t = sxv[vox * 3 + ch] * inv;
      }
      se[(s * kOwn + q) * 3 + ch] = t;
    }
  }
}

// inference input: wx[b][v][ch] = dinv .* v on R around mesh block b
__global__ void __launch_bounds__(256) k_gather_region(int nb, long long nvc,
                                                       const int* __restrict__ in_map,
                                                       const int* __restrict__ hs,
                                                       const int* __restrict__ hp,
                                                       const double* __restrict__ hw,
                                                       const double* __restrict__ vin,
                                                       const double* __restrict__ dinv,
                                                       float* __restrict__ wx) {
  const int b = blockIdx.x;
  for (int q = threadIdx.x; q < kRV; q += blockDim.x) {
    const int id = in_map[(size_t)b * kRV + q];
#pragma unroll
    for (int ch = 0; ch < 3; ch++)
      wx[((size_t)b * kRV + q) * 3 + ch] = (float)pc_input(id, ch, nvc, vin, dinv, hs, hp, hw);
  }
}

// z (FP64) = x + y on the corners block b writes, for the blocks of weight set
// `want` (all blocks when set is null)
__global__ void __launch_bounds__(256) k_scatter_z(int nb, long long nvc,
                                                   const int* __restrict__ out_map,
                                                   const int* __restrict__ set, int want,
                                                   const float* __restrict__ wx,
                                                   const float* __restrict__ y,
                                                   double* __restrict__ z) {
  const int b = blockIdx.x;
  if (set && set[b] != want) return;
  for (int q = threadIdx.x; q < kOwn; q += blockDim.x) {
    const int id = out_map[(size_t)b * kOwn + q];
    if (id < 0) continue;
    const int i = q & 7, j = (q >> 3) & 7, k = q >> 6;
    const int v = ((k + 1) * 10 + (j + 1)) * 10 + (i + 1);
#pragma unroll
    for (int ch = 0; ch < 3; ch++)
      z[ch * nvc + id] = (double)(wx[((size_t)b * kRV + v) * 3 + ch] + y[((size_t)b * kRV + v) * 3 + ch]);
  }
}

// z = dinv .* v on the corners no block writes (hanging corners)
__global__ void __launch_bounds__(256) k_pc_jacobi(long long n, const int* __restrict__ ids,
                                                   long long nvc, const double* __restrict__ vin,
                                                   const double* __restrict__ dinv,
                                                   double* __restrict__ z) {
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const long long id = ids[q];
#pragma unroll
    for (int ch = 0; ch < 3; ch++) z[ch * nvc + id] = dinv[ch * nvc + id] * vin[ch * nvc + id];
  }
}

// region-layout y -> owned [s][512][3]
__global__ void k_owned_out(int S, const float* __restrict__ y, float* __restrict__ out) {
  const int s = blockIdx.x;
  for (int q = threadIdx.x; q < kOwn; q += blockDim.x) {
    const int i = q & 7, j = (q >> 3) & 7, k = q >> 6;
    const int v = ((k + 1) * 10 + (j + 1)) * 10 + (i + 1);
#pragma unroll
    for (int ch = 0; ch < 3; ch++)
      out[((size_t)s * kOwn + q) * 3 + ch] = y[((size_t)s * kRV + v) * 3 + ch];
  }
}

template <int CIN, int COUT>
size_t conv_smem() {
  return sizeof(float) * (27 * CIN * COUT + 300 * (CIN + 1));
}

template <int CIN, int COUT>
cudaError_t conv(PrecondState* P, cudaStream_t st, int S, const float* in, const float* W,
                 float* out, int owned_only) {
  const size_t sm = conv_smem<CIN, COUT>();
  static unsigned long long attr_set = 0;  // per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (!((attr_set >> dev) & 1ull)) {
    cudaFuncSetAttribute(k_conv<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    attr_set |= 1ull << dev;
  }
  k_conv<CIN, COUT><<<dim3(kR, S), 256, sm, st>>>(in, W, out, owned_only);
  return cudaGetLastError();
}

template <int CIN, int COUT>
cudaError_t wgrad(cudaStream_t st, int S, const float* dout, const float* in, float* dW) {
  const int chunk = 4;
  k_wgrad<CIN, COUT><<<dim3(27, (S + chunk - 1) / chunk), 256, 0, st>>>(S, chunk, dout, in, dW);
  return cudaGetLastError();
}

}  // namespace

// ===========================================================================
const int kWSize[3] = {27 * 3 * 32, 27 * 32 * 32, 27 * 32 * 3};

static void free_work(PrecondState* P) {
  float* ws[] = {P->wx, P->we, P->h1, P->h2, P->y, P->dy, P->dh1, P->dh2, P->wt};
  for (float* p : ws) cudaFree(p);
  cudaFree(P->perm);
  P->wx = P->we = P->h1 = P->h2 = P->y = P->dy = P->dh1 = P->dh2 = P->wt = nullptr;
  P->perm = nullptr;
  P->work_S = 0;
}

cudaError_t precond_work(PrecondState* P, int S) {
  if (P->work_S >= S) return cudaSuccess;
  free_work(P);
  cudaError_t e = cudaSuccess;
  auto al = [&](float** p, size_t n) {
    if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(p), sizeof(float) * n);
  };
  al(&P->wx, (size_t)S * kRV * 3);
  al(&P->we, (size_t)S * kOwn * 3);
  al(&P->h1, (size_t)S * kRV * 32);
  al(&P->h2, (size_t)S * kRV * 32);
  al(&P->y, (size_t)S * kRV * 3);
  al(&P->dy, (size_t)S * kRV * 3);
  al(&P->dh1, (size_t)S * kRV * 32);
  al(&P->dh2, (size_t)S * kRV * 32);
  al(&P->wt, (size_t)27 * 32 * 32);
  if (e == cudaSuccess) P->work_S = S;
  return e;
}

void precond_select(PrecondState* P, int set) {
  P->adam_saved[(size_t)P->active] = P->adam_t;
  P->active = set;
  for (int l = 0; l < 3; l++) {
    const size_t o = (size_t)set * kWSize[l];
    P->w[l] = P->wb[l] + o;
    P->g[l] = P->gb[l] + o;
    P->m[l] = P->mb[l] + o;
    P->v[l] = P->vb[l] + o;
  }
  P->adam_t = P->adam_saved[(size_t)set];
}

void precond_free(PrecondState* P) {
  if (!P) return;
  free_work(P);
  for (int l = 0; l < 3; l++) {
    cudaFree(P->wb[l]); cudaFree(P->gb[l]); cudaFree(P->mb[l]); cudaFree(P->vb[l]);
  }
  cudaFree(P->wtc);
  cudaFree(P->dloss);
  cudaFree(P->sx);
  cudaFree(P->se);
  delete P;
}

// forward of the FP32 training path: wx -> h1 -> h2 -> y (owned voxels)
cudaError_t precond_forward32(PrecondState* P, cudaStream_t st, int S) {
  cudaError_t e;
  if ((e = conv<3, 32>(P, st, S, P->wx, P->w[0], P->h1, 0)) != cudaSuccess) return e;
  if ((e = conv<32, 32>(P, st, S, P->h1, P->w[1], P->h2, 0)) != cudaSuccess) return e;
  return conv<32, 3>(P, st, S, P->h2, P->w[2], P->y, 1);
}

// loss (added into *d_loss) and weight gradients (added into g) of the batch in wx/we
cudaError_t precond_backward32(PrecondState* P, cudaStream_t st, int S, double* d_loss) {
  cudaError_t e;
  if ((e = precond_forward32(P, st, S)) != cudaSuccess) return e;
  k_loss<<<std::min(S * 4, 1024), 256, 0, st>>>(S, P->wx, P->y, P->we, P->dy, d_loss);
  if ((e = wgrad<32, 3>(st, S, P->dy, P->h2, P->g[2])) != cudaSuccess) return e;
  k_flip<<<64, 256, 0, st>>>(P->w[2], P->wt, 32, 3);
  if ((e = conv<3, 32>(P, st, S, P->dy, P->wt, P->dh2, 0)) != cudaSuccess) return e;
  if ((e = wgrad<32, 32>(st, S, P->dh2, P->h1, P->g[1])) != cudaSuccess) return e;
  k_flip<<<64, 256, 0, st>>>(P->w[1], P->wt, 32, 32);
  if ((e = conv<32, 32>(P, st, S, P->dh2, P->wt, P->dh1, 0)) != cudaSuccess) return e;
  return wgrad<3, 32>(st, S, P->dh1, P->wx, P->g[0]);
}

cudaError_t precond_zero_grads(PrecondState* P, cudaStream_t st) {
  for (int l = 0; l < 3; l++) {
    cudaError_t e = cudaMemsetAsync(P->g[l], 0, sizeof(float) * kWSize[l], st);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t precond_adam(PrecondState* P, cudaStream_t st, float lr) {
  P->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.0f / (1.0f - std::pow(b1, (float)P->adam_t));
  const float c2 = 1.0f / (1.0f - std::pow(b2, (float)P->adam_t));
  for (int l = 0; l < 3; l++)
    k_adam<<<64, 256, 0, st>>>(kWSize[l], P->w[l], P->g[l], P->m[l], P->v[l], lr, b1, b2, c1, c2,
                               1e-8f);
  return cudaGetLastError();
}

cudaError_t precond_gather_batch(PrecondState* P, cudaStream_t st, int S, long long first) {
  k_gather_batch<<<S, 256, 0, st>>>(S, P->perm, first, P->sx, P->se, P->wx, P->we);
  return cudaGetLastError();
}

cudaError_t precond_harvest_pairs(amps_gpu_ctx* c, const double* r, const double* e, int e_scaled) {
  PrecondState* P = c->pn;
  if (!P || P->cap <= 0 || P->n >= P->cap || !c->d_dinv) return cudaSuccess;
  TimedLaunch t(c, "precond_harvest");
  k_harvest<<<c->nb, 256, 0, c->stream>>>(c->nb, c->nvc, c->d_pc_in, c->d_hs, c->d_hp, c->d_hw,
                                          c->d_pc_out_v[0], r, e, c->d_dinv,
                                          e_scaled, P->sx, P->se, P->n, P->cap);
  const long long add = std::min<long long>(P->cap - P->n, c->nb);
  P->sample_set.insert(P->sample_set.end(), c->h_pc_set.begin(), c->h_pc_set.begin() + add);
  P->sample_iface.insert(P->sample_iface.end(), c->h_pc_iface.begin(), c->h_pc_iface.begin() + add);
  P->n += add;
  return cudaGetLastError();
}

// z = D v + N(D v) on the mesh
cudaError_t launch_precond_net(amps_gpu_ctx* c, const double* v, double* z) {
  PrecondState* P = c->pn;
  if (!P) return cudaErrorInvalidValue;
  cudaError_t e;
  if (c->pc_njac > 0) {
    TimedLaunch t(c, "precond_jacobi_hanging");
    k_pc_jacobi<<<(unsigned)std::min<long long>((c->pc_njac + 255) / 256, 1216), 256, 0, c->stream>>>(
        c->pc_njac, c->d_pc_jac, c->nvc, v, c->d_dinv, z);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (P->use_tc) {
    TimedLaunch t(c, "precond_net_tc");
    return precond_apply_tc_mesh(P, c->stream, c->nb, c->d_pc_in, c->d_hs, c->d_hp, c->d_hw,
                                 c->d_pc_out, c->d_pc_set, c->nvc, v, c->d_dinv, z);
  }
  if ((e = precond_work(P, c->nb)) != cudaSuccess) return e;
  {
    TimedLaunch t(c, "precond_gather");
    k_gather_region<<<c->nb, 256, 0, c->stream>>>(c->nb, c->nvc, c->d_pc_in, c->d_hs, c->d_hp,
                                                  c->d_hw, v, c->d_dinv, P->wx);
  }
  // the FP32 path runs every set's network over all blocks and keeps each
  // block's own
  const int active = P->active;
  for (int s = 0; s < P->nsets; s++) {
    precond_select(P, s);
    {
      TimedLaunch t(c, "precond_net_fp32", 3);
      if ((e = precond_forward32(P, c->stream, c->nb)) != cudaSuccess) break;
    }
    TimedLaunch t(c, "precond_scatter");
    k_scatter_z<<<c->nb, 256, 0, c->stream>>>(c->nb, c->nvc, c->d_pc_out, c->d_pc_set, s, P->wx,
                                              P->y, z);
  }
  precond_select(P, active);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

cudaError_t precond_owned_out(PrecondState* P, cudaStream_t st, int S, float* out) {
  k_owned_out<<<S, 256, 0, st>>>(S, P->y, out);
  return cudaGetLastError();
}

// ===========================================================================
// C ABI
namespace {

amps_gpu_status ensure_state(amps_gpu_ctx* c) {
  if (c->pn) return AMPS_GPU_OK;
  PrecondState* P = new PrecondState();
  P->nsets = c->pc_nsets;
  P->adam_saved.assign((size_t)P->nsets, 0);
  bool ok = true;
  for (int l = 0; l < 3 && ok; l++) {
    const size_t bytes = sizeof(float) * kWSize[l] * (size_t)P->nsets;
    for (float** p : {&P->wb[l], &P->gb[l], &P->mb[l], &P->vb[l]}) {
      ok = ok && cudaMalloc(reinterpret_cast<void**>(p), bytes) == cudaSuccess;
      ok = ok && cudaMemset(*p, 0, bytes) == cudaSuccess;
    }
  }
  if (ok) precond_select(P, 0);
  ok = ok && cudaMalloc(reinterpret_cast<void**>(&P->dloss), sizeof(double) * 4) == cudaSuccess;
  if (!c->d_Z)
    ok = ok && cudaMalloc(reinterpret_cast<void**>(&c->d_Z),
                          sizeof(double) * (size_t)(c->restart + 1) * 3 * c->nvc) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    precond_free(P);
    return set_err(c, AMPS_GPU_CUDA_ERROR, "learned preconditioner: allocation failed");
  }
  P->flags = c->d_flags;
  // BF16 images of every set (zero weights: the network adds nothing)
  for (int s = 0; s < P->nsets && ok; s++) {
    precond_select(P, s);
    ok = precond_prepare_tc(P, c->stream) == cudaSuccess;
  }
  if (ok) precond_select(P, 0);
  ok = ok && cudaStreamSynchronize(c->stream) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    precond_free(P);
    return set_err(c, AMPS_GPU_CUDA_ERROR, "learned preconditioner: weight images");
  }
  c->pn = P;
  return AMPS_GPU_OK;
}

amps_gpu_status upload_samples(amps_gpu_ctx* c, long long count, const float* x, const float* e) {
  PrecondState* P = c->pn;
  cudaError_t er = precond_work(P, (int)count);
  if (er != cudaSuccess) return cuda_check(c, er, "precond work buffers");
  er = cudaMemcpy(P->wx, x, sizeof(float) * count * 1000 * 3, cudaMemcpyHostToDevice);
  if (er == cudaSuccess && e)
    er = cudaMemcpy(P->we, e, sizeof(float) * count * 512 * 3, cudaMemcpyHostToDevice);
  return cuda_check(c, er, "upload samples");
}

}  // namespace

extern "C" {

amps_gpu_status amps_gpu_set_inner_fp64(amps_gpu_ctx* c, int fp64) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  c->inner_fp32 = fp64 == 0;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_precond_load(amps_gpu_ctx* c, const float* w1, const float* w2,
                                      const float* w3) {
  if (!c || !w1 || !w2 || !w3) return set_err(c, AMPS_GPU_INVALID_ARG, "precond_load: null weights");
  cudaSetDevice(c->cfg.device);
  amps_gpu_status s = ensure_state(c);
  if (s) return s;
  PrecondState* P = c->pn;
  const float* src[3] = {w1, w2, w3};
  cudaStreamSynchronize(c->stream);
  for (int l = 0; l < 3; l++) {
    if ((s = cuda_check(c, cudaMemcpy(P->w[l], src[l], sizeof(float) * kWSize[l], cudaMemcpyHostToDevice),
                        "upload weights")))
      return s;
    cudaMemset(P->m[l], 0, sizeof(float) * kWSize[l]);
    cudaMemset(P->v[l], 0, sizeof(float) * kWSize[l]);
  }
  P->adam_t = 0;
  P->tc_ready = false;
  return cuda_check(c, precond_prepare_tc(P, c->stream), "prepare tensor-core weights");
}

amps_gpu_status amps_gpu_precond_use_tensor_cores(amps_gpu_ctx* c, int on) {
  if (!c || !c->pn) return set_err(c, AMPS_GPU_INVALID_ARG, "precond_use_tensor_cores: no network");
  if (on && !c->pn->tc_ready)
    return set_err(c, AMPS_GPU_INVALID_ARG, "precond_use_tensor_cores: weights not prepared");
  c->pn->use_tc = on != 0;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_precond_get(amps_gpu_ctx* c, float* w1, float* w2, float* w3) {
  if (!c || !c->pn) return set_err(c, AMPS_GPU_INVALID_ARG, "precond_get: no network");
  cudaSetDevice(c->cfg.device);
  cudaStreamSynchronize(c->stream);
  float* dst[3] = {w1, w2, w3};
  for (int l = 0; l < 3; l++)
    if (dst[l]) {
      amps_gpu_status s = cuda_check(
          c, cudaMemcpy(dst[l], c->pn->w[l], sizeof(float) * kWSize[l], cudaMemcpyDeviceToHost),
          "download weights");
      if (s) return s;
    }
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_precond_harvest(amps_gpu_ctx* c, long long capacity) {
  if (!c || capacity < 0) return set_err(c, AMPS_GPU_INVALID_ARG, "precond_harvest: bad capacity");
  cudaSetDevice(c->cfg.device);
  amps_gpu_status s = ensure_state(c);
  if (s) return s;
  PrecondState* P = c->pn;
  cudaStreamSynchronize(c->stream);
  cudaFree(P->sx);
  cudaFree(P->se);
  P->sx = P->se = nullptr;
  P->cap = P->n = 0;
  P->sample_set.clear();
  P->sample_iface.clear();
  if (capacity == 0) return AMPS_GPU_OK;
  if (cudaMalloc(reinterpret_cast<void**>(&P->sx), sizeof(float) * capacity * 1000 * 3) != cudaSuccess ||
      cudaMalloc(reinterpret_cast<void**>(&P->se), sizeof(float) * capacity * 512 * 3) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(P->sx);
    P->sx = nullptr;
    return set_err(c, AMPS_GPU_CUDA_ERROR, "precond_harvest: allocation failed");
  }
  P->cap = capacity;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_precond_num_sets(amps_gpu_ctx* c, int* n) {
  if (!c || !n) return AMPS_GPU_INVALID_ARG;
  *n = c->pc_nsets;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_precond_select(amps_gpu_ctx* c, int set) {
  if (!c || set < 0 || set >= c->pc_nsets)
    return set_err(c, AMPS_GPU_INVALID_ARG, "precond_select: no such weight set");
  cudaSetDevice(c->cfg.device);
  amps_gpu_status s = ensure_state(c);
  if (s) return s;
  precond_select(c->pn, set);
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_precond_interface_jacobi(amps_gpu_ctx* c, int on, int* nblocks) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  const int q = on ? 1 : 0;
  c->pc_iface_jacobi = on != 0;
  c->d_pc_out = c->d_pc_out_v[q];
  c->d_pc_jac = c->d_pc_jac_v[q];
  c->pc_njac = c->pc_njac_v[q];
  if (nblocks) *nblocks = c->pc_iface_blocks;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_precond_sample_sets(amps_gpu_ctx* c, long long first, long long count,
                                             int32_t* sets) {
  if (!c || !c->pn || !sets || first < 0 || count < 0 || first + count > c->pn->n)
    return set_err(c, AMPS_GPU_INVALID_ARG, "precond_sample_sets: range");
  for (long long q = 0; q < count; q++) sets[q] = c->pn->sample_set[(size_t)(first + q)];
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_precond_num_samples(amps_gpu_ctx* c, long long* n) {
  if (!c || !n) return AMPS_GPU_INVALID_ARG;
  *n = c->pn ? c->pn->n : 0;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_precond_get_samples(amps_gpu_ctx* c, long long first, long long count,
                                             float* x, float* e) {
  if (!c || !c->pn || first < 0 || count < 0 || first + count > c->pn->n)
    return set_err(c, AMPS_GPU_INVALID_ARG, "precond_get_samples: range");
  cudaSetDevice(c->cfg.device);
  cudaStreamSynchronize(c->stream);
  PrecondState* P = c->pn;
  cudaError_t er = cudaSuccess;
  if (x) er = cudaMemcpy(x, P->sx + first * 3000, sizeof(float) * count * 3000, cudaMemcpyDeviceToHost);
  if (er == cudaSuccess && e)
    er = cudaMemcpy(e, P->se + first * 1536, sizeof(float) * count * 1536, cudaMemcpyDeviceToHost);
  return cuda_check(c, er, "download samples");
}

amps_gpu_status amps_gpu_precond_train(amps_gpu_ctx* c, int epochs, int batch, float lr,
                                       unsigned long long seed, float* loss_out) {
  if (!c || !c->pn || epochs <= 0 || batch <= 0 || !(lr > 0.f))
    return set_err(c, AMPS_GPU_INVALID_ARG, "precond_train: bad arguments");
  PrecondState* P = c->pn;
  // the active set's samples (without those of interface blocks when these
  // use Jacobi)
  std::vector<int> perm;
  for (long long q = 0; q < P->n; q++)
    if (P->sample_set[(size_t)q] == P->active && !(c->pc_iface_jacobi && P->sample_iface[(size_t)q]))
      perm.push_back((int)q);
  const long long ns = (long long)perm.size();
  if (ns < 1) return set_err(c, AMPS_GPU_INVALID_ARG, "precond_train: no samples of this weight set");
  cudaSetDevice(c->cfg.device);
  cudaStream_t st = c->stream;
  const int S = (int)std::min<long long>(batch, ns);
  cudaError_t er = precond_work(P, S);
  if (er != cudaSuccess) return cuda_check(c, er, "precond work buffers");
  if (P->perm_n < ns) {
    cudaFree(P->perm);
    if (cudaMalloc(reinterpret_cast<void**>(&P->perm), sizeof(int) * ns) != cudaSuccess)
      return set_err(c, AMPS_GPU_CUDA_ERROR, "precond_train: allocation failed");
    P->perm_n = ns;
  }
  std::mt19937_64 rng(seed);
  const long long nbatch = ns / S;
  const double total = (double)epochs * (double)nbatch;
  long long step = 0;
  for (int ep = 0; ep < epochs; ep++) {
    std::shuffle(perm.begin(), perm.end(), rng);
    er = cudaMemcpyAsync(P->perm, perm.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, st);
    if (er == cudaSuccess) er = cudaMemsetAsync(P->dloss, 0, sizeof(double), st);
    for (long long bi = 0; bi < nbatch && er == cudaSuccess; bi++) {
      TimedLaunch t(c, "precond_train", 12);
      if ((er = precond_gather_batch(P, st, S, bi * S)) != cudaSuccess) break;
      if ((er = precond_zero_grads(P, st)) != cudaSuccess) break;
      if ((er = precond_backward32(P, st, S, P->dloss)) != cudaSuccess) break;
      // cosine decay of the learning rate to 1% over the run
      const double ph = (double)(step++) / total;
      er = precond_adam(P, st, (float)(lr * (0.01 + 0.99 * 0.5 * (1.0 + std::cos(3.14159265358979 * ph)))));
    }
    double lsum = 0.0;
    if (er == cudaSuccess)
      er = cudaMemcpyAsync(&lsum, P->dloss, sizeof(double), cudaMemcpyDeviceToHost, st);
    if (er == cudaSuccess) er = cudaStreamSynchronize(st);
    if (er != cudaSuccess) return cuda_check(c, er, "precond_train");
    if (loss_out) loss_out[ep] = (float)(lsum / (double)nbatch);
  }
  P->tc_ready = false;
  return cuda_check(c, precond_prepare_tc(P, st), "prepare tensor-core weights");
}

amps_gpu_status amps_gpu_precond_loss_grad(amps_gpu_ctx* c, long long count, const float* x,
                                           const float* e, float* loss, float* g1, float* g2,
                                           float* g3) {
  if (!c || !c->pn || count <= 0 || !x || !e)
    return set_err(c, AMPS_GPU_INVALID_ARG, "precond_loss_grad: bad arguments");
  cudaSetDevice(c->cfg.device);
  PrecondState* P = c->pn;
  cudaStreamSynchronize(c->stream);
  amps_gpu_status s = upload_samples(c, count, x, e);
  if (s) return s;
  cudaStream_t st = c->stream;
  cudaError_t er = precond_zero_grads(P, st);
  if (er == cudaSuccess) er = cudaMemsetAsync(P->dloss, 0, sizeof(double), st);
  if (er == cudaSuccess) er = precond_backward32(P, st, (int)count, P->dloss);
  double l = 0.0;
  if (er == cudaSuccess) er = cudaMemcpyAsync(&l, P->dloss, sizeof(double), cudaMemcpyDeviceToHost, st);
  if (er == cudaSuccess) er = cudaStreamSynchronize(st);
  float* dst[3] = {g1, g2, g3};
  for (int q = 0; q < 3 && er == cudaSuccess; q++)
    if (dst[q]) er = cudaMemcpy(dst[q], P->g[q], sizeof(float) * kWSize[q], cudaMemcpyDeviceToHost);
  if (er != cudaSuccess) return cuda_check(c, er, "precond_loss_grad");
  if (loss) *loss = (float)l;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_precond_forward(amps_gpu_ctx* c, long long count, const float* x,
                                         int tensor_cores, float* y) {
  if (!c || !c->pn || count <= 0 || !x || !y)
    return set_err(c, AMPS_GPU_INVALID_ARG, "precond_forward: bad arguments");
  cudaSetDevice(c->cfg.device);
  PrecondState* P = c->pn;
  cudaStreamSynchronize(c->stream);
  amps_gpu_status s = upload_samples(c, count, x, nullptr);
  if (s) return s;
  cudaStream_t st = c->stream;
  cudaError_t er;
  if (tensor_cores) {
    if (!P->tc_ready) return set_err(c, AMPS_GPU_INVALID_ARG, "precond_forward: tensor-core path not ready");
    TimedLaunch t(c, "precond_forward_tc");
    er = precond_forward_tc(P, st, (int)count, P->wx, P->y);
  } else {
    TimedLaunch t(c, "precond_forward_fp32", 3);
    er = precond_forward32(P, st, (int)count);
  }
  if (er == cudaSuccess) er = precond_owned_out(P, st, (int)count, P->dh1);
  if (er == cudaSuccess) er = cudaStreamSynchronize(st);
  if (er == cudaSuccess)
    er = cudaMemcpy(y, P->dh1, sizeof(float) * count * 512 * 3, cudaMemcpyDeviceToHost);
  return cuda_check(c, er, "precond_forward");
}

}  // extern "C"
