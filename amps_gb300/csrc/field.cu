// ECSIM field solve on sm_103a on uniform meshes (FP64 vectors; the inner
// GMRES operator in FP32 arithmetic around an FP64 identity part).
//
//   k_rhs       UpdateRhs with the supports registered by GetStencil
//               (src/pic/ecsim/get_stencil.cpp:1260-1599, ecsim/update_rhs.cpp:285):
//               theta c dt curl B^n - 4 pi theta dt J - (theta c dt)^2 curlcurl E^n
//               - 4 pi theta dt M E^n
//   k_matvec    the assembled row of GetStencil valued by UpdateMatrixElement
//               (pic_field_solver_ecsim.cpp:6004-6019) applied matrix-free:
//               A = I + (theta c dt)^2 (grad div - lap) + 4 pi theta dt M
//               (replaces cLinearSystemCornerNode::MultiplyVector,
//               srcInterface/LinearSystemCornerNode.h:3067-3205)
//   GMRES       restarted GMRES(30), x0 = 0, right preconditioner (none,
//               Jacobi, learned), classical Gram-Schmidt with one
//               re-orthogonalisation; each Arnoldi step is matvec + three fused
//               sweep/reduction kernels with FP64 warp-shuffle reductions
//               (the external linear_solver_wrapper of LinearSystemCornerNode.h:3282)
//   k_update_b  UpdateB (:5160-5711), k_c2n InterpolateB_C2N (:5715),
//   k_update_e  UpdateE with the wave-energy sum (:5909-6001)
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "precond.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr int kMaxV = 32;
constexpr int kRedBlocks = 304;  // 2 x 152 SMs
constexpr int kGmOffset = 10240;  // doubles into d_red (12288 doubles)
constexpr int kArnMaxGrid = 1024;  // CTAs of the cooperative Arnoldi step (at most)

struct Taps {
  double K[3][3][27];  // operator taps without the mass matrix
  double f;            // 4 pi theta dt
};

double tap_s(int o) { return o == 0 ? 0.5 : 0.25; }
double tap_d2(int o) { return o == 0 ? -2.0 : 1.0; }
double tap_d1(int o) { return o == 0 ? 0.0 : (o > 0 ? 0.5 : -0.5); }

// Separable form of the compact stencils built by InitDiscritizationStencil
// (pic_field_solver_ecsim.cpp:7121): d2/dx2 = D2(x) S(y) S(z),
// d2/dxdy = D1(x) D1(y) S(z), with S = (1/4, 1/2, 1/4), D2 = (1,-2,1), D1 = (-1/2,0,1/2).
Taps make_taps(const amps_gpu_config& cfg, bool identity) {
  Taps t{};
  double coeff[3], cs[3];
  for (int d = 0; d < 3; d++) {
    coeff[d] = cfg.dt / cfg.dx[d] * cfg.theta;
    cs[d] = coeff[d] * coeff[d];
  }
  for (int dk = -1; dk <= 1; dk++)
    for (int dj = -1; dj <= 1; dj++)
      for (int di = -1; di <= 1; di++) {
        const int o[3] = {di, dj, dk};
        const int s = mm_slot(di, dj, dk);
        double lap[3];
        for (int ax = 0; ax < 3; ax++) {
          double a = 1.0;
          for (int d = 0; d < 3; d++) a *= (d == ax) ? tap_d2(o[d]) : tap_s(o[d]);
          lap[ax] = a;
        }
        for (int p = 0; p < 3; p++)
          for (int q = 0; q < 3; q++) {
            double gd;
            if (p == q) {
              gd = lap[p];
            } else {
              gd = 1.0;
              for (int d = 0; d < 3; d++) gd *= (d == p || d == q) ? tap_d1(o[d]) : tap_s(o[d]);
            }
            double a = 0.0;
            if (p == q) {
              for (int d = 0; d < 3; d++) a -= lap[d] * cs[d];
              if (s == 0 && identity) a += 1.0;
            }
            a += gd * coeff[p] * coeff[q];
            t.K[p][q][s] = a;
          }
      }
  t.f = 4.0 * kPi * cfg.dt * cfg.theta;
  return t;
}

__device__ __forceinline__ void corner_ijk(long long c, int& b, int& i, int& j, int& k) {
  b = (int)(c / AMPS_CPB);
  const int l = (int)(c % AMPS_CPB);
  i = l & 7;
  j = (l >> 3) & 7;
  k = l >> 6;
}

// The operator taps split into FP32 pairs (K = Kh + Kl) for the FP64-accurate
// evaluations below.
struct TapsFF {
  float Kh[3][3][27], Kl[3][3][27];
  double f;
};

TapsFF taps_ff(const Taps& T) {
  TapsFF t;
  for (int p = 0; p < 3; p++)
    for (int q = 0; q < 3; q++)
      for (int s = 0; s < 27; s++) {
        t.Kh[p][q][s] = (float)T.K[p][q][s];
        t.Kl[p][q][s] = (float)(T.K[p][q][s] - (double)t.Kh[p][q][s]);
      }
  t.f = T.f;
  return t;
}

// xh + xl = dinv .* x (dinv may be null), split into FP32 pairs (xl null: the
// FP32 rounding only, the input of the FP32 inner operator)
__global__ void __launch_bounds__(256) k_split(long long n, const double* __restrict__ x,
                                               const double* __restrict__ dinv,
                                               float* __restrict__ xh, float* __restrict__ xl) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const double v = dinv ? dinv[t] * x[t] : x[t];
    const float h = (float)v;
    xh[t] = h;
    if (xl) xl[t] = (float)(v - (double)h);
  }
}

// Row (p, corner c) of (K + f M) x to FP64 accuracy: the 27-point taps and
// the corner's 243 FP32 mass-matrix coefficients against the split input.
__device__ __forceinline__ double row_ff(long long ncor, const int* __restrict__ nbr,
                                         const float* __restrict__ M, const float* __restrict__ xh,
                                         const float* __restrict__ xl, const TapsFF& T, int p,
                                         long long c, int b, int i, int j, int k) {
  FF sk{0.f, 0.f}, sm{0.f, 0.f};
#pragma unroll 3
  for (int s = 0; s < 27; s++) {
    const int dig[3] = {s % 3, (s / 3) % 3, s / 9};
    const int di = dig[0] == 0 ? 0 : (dig[0] == 1 ? -1 : 1);
    const int dj = dig[1] == 0 ? 0 : (dig[1] == 1 ? -1 : 1);
    const int dk = dig[2] == 0 ? 0 : (dig[2] == 1 ? -1 : 1);
    const int nb = local_id(nbr, b, i + di, j + dj, k + dk);
    const float* Ms = M + (size_t)(9 * s + 3 * p) * ncor + c;
#pragma unroll
    for (int q = 0; q < 3; q++) {
      const float h = xh[q * ncor + nb], lo = xl[q * ncor + nb];
      ff_add2(sk, T.Kh[p][q][s], T.Kl[p][q][s], h, lo);
      ff_add(sm, Ms[(size_t)q * ncor], h, lo);
    }
  }
  return ff_value(sk) + T.f * ff_value(sm);
}

// y = A (dinv .* x) to FP64 accuracy from the split input (outer residuals);
// one thread per (component p, corner)
__global__ void __launch_bounds__(256) k_matvec(long long ncor, const int* __restrict__ nbr,
                                                const float* __restrict__ M,
                                                const float* __restrict__ xh,
                                                const float* __restrict__ xl,
                                                double* __restrict__ y, TapsFF T) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * ncor) return;
  const int p = (int)(t / ncor);
  const long long c = t - (long long)p * ncor;
  int b, i, j, k;
  corner_ijk(c, b, i, j, k);
  y[t] = row_ff(ncor, nbr, M, xh, xl, T, p, c, b, i, j, k);
}

struct TapsF {
  float K[3][3][27];
  float f;
};

TapsF taps_f32(const Taps& T) {
  TapsF t;
  for (int p = 0; p < 3; p++)
    for (int q = 0; q < 3; q++)
      for (int s = 0; s < 27; s++) t.K[p][q][s] = (float)T.K[p][q][s];
  t.f = (float)T.f;
  return t;
}

// y = A (dinv .* x) with the identity part in FP64 and the rest (curl-curl
// and mass-matrix terms, a small fraction of A on ECSIM time steps) in FP32
// arithmetic: the inner operator of the refined GMRES, which never decides
// convergence.  One thread per (component p, corner).
__global__ void __launch_bounds__(256) k_matvec32(long long ncor, const int* __restrict__ nbr,
                                                  const float* __restrict__ M,
                                                  const float* __restrict__ xf,
                                                  const double* __restrict__ x,
                                                  const double* __restrict__ dinv,
                                                  double* __restrict__ y, TapsF T) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * ncor) return;
  const int p = (int)(t / ncor);
  const long long c = t - (long long)p * ncor;
  int b, i, j, k;
  corner_ijk(c, b, i, j, k);
  float acc = 0.f;
#pragma unroll 3
  for (int s = 0; s < 27; s++) {
    const int dig[3] = {s % 3, (s / 3) % 3, s / 9};
    const int di = dig[0] == 0 ? 0 : (dig[0] == 1 ? -1 : 1);
    const int dj = dig[1] == 0 ? 0 : (dig[1] == 1 ? -1 : 1);
    const int dk = dig[2] == 0 ? 0 : (dig[2] == 1 ? -1 : 1);
    const int nb = local_id(nbr, b, i + di, j + dj, k + dk);
    const float* Ms = M + (size_t)(9 * s + 3 * p) * ncor + c;
#pragma unroll
    for (int q = 0; q < 3; q++)
      acc = fmaf(fmaf(T.f, Ms[(size_t)q * ncor], T.K[p][q][s]), xf[q * ncor + nb], acc);
  }
  const double xi = dinv ? dinv[t] * x[t] : x[t];
  y[t] = xi + (double)acc;
}

// RHS: theta c dt curl B^n - f J - (curl-curl + f M) E^n, the last term to
// FP64 accuracy from the split E^n (taps without the identity)
__global__ void __launch_bounds__(256) k_rhs(long long ncor, const int* __restrict__ nbr,
                                             const float* __restrict__ M,
                                             const float* __restrict__ Eh,
                                             const float* __restrict__ El,
                                             const double* __restrict__ Bc,
                                             const double* __restrict__ J,
                                             double* __restrict__ rhs, TapsFF T, double c4x,
                                             double c4y, double c4z) {
  // one thread per (component p, corner)
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * ncor) return;
  const int p = (int)(t / ncor);
  const long long c = t - (long long)p * ncor;
  int b, i, j, k;
  corner_ijk(c, b, i, j, k);
  double r = -row_ff(ncor, nbr, M, Eh, El, T, p, c, b, i, j, k);
  r -= T.f * J[t];
  // curl B^n from the 2x2 face averages of the 8 cells around the corner
  auto Bv = [&](int ii, int jj, int kk, int comp) {
    return Bc[comp * ncor + local_id(nbr, b, ii, jj, kk)];
  };
  double cb = 0.0;
  for (int a = -1; a <= 0; a++)
    for (int q = -1; q <= 0; q++) {
      if (p == 0) {
        cb += c4y * (Bv(i + a, j, k + q, 2) - Bv(i + a, j - 1, k + q, 2));
        cb += -c4z * (Bv(i + a, j + q, k, 1) - Bv(i + a, j + q, k - 1, 1));
      } else if (p == 1) {
        cb += c4z * (Bv(i + a, j + q, k, 0) - Bv(i + a, j + q, k - 1, 0));
        cb += -c4x * (Bv(i, j + q, k + a, 2) - Bv(i - 1, j + q, k + a, 2));
      } else {
        cb += c4x * (Bv(i, j + q, k + a, 1) - Bv(i - 1, j + q, k + a, 1));
        cb += -c4y * (Bv(i + q, j, k + a, 0) - Bv(i + q, j - 1, k + a, 0));
      }
    }
  rhs[t] = r + cb;
}

__global__ void __launch_bounds__(256) k_jacobi(long long ncor, const float* __restrict__ M,
                                                double* __restrict__ dinv, double k00, double k11,
                                                double k22, double f) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncor) return;
  // a preconditioner: FP32 arithmetic (FP64 division is slow on this part)
  dinv[c] = (double)(1.0f / fmaf((float)f, M[(size_t)0 * ncor + c], (float)k00));
  dinv[ncor + c] = (double)(1.0f / fmaf((float)f, M[(size_t)4 * ncor + c], (float)k11));
  dinv[2 * ncor + c] = (double)(1.0f / fmaf((float)f, M[(size_t)8 * ncor + c], (float)k22));
}

// ---- reductions ------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Reduce acc[0..nv) over the block and store partial[blockIdx.x*kMaxV + i].
template <int NVM>
__device__ __forceinline__ void block_store_partials(double* acc, int nv, double* partial) {
  __shared__ double s_red[8][NVM];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NVM; i++) {
    if (i < nv) {
      double v = warp_sum(acc[i]);
      if (lane == 0) s_red[wid][i] = v;
    }
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_red[w][threadIdx.x];
    partial[blockIdx.x * kMaxV + threadIdx.x] = t;
  }
}

__global__ void k_reduce_partials(const double* __restrict__ partial, int nblk, int nv,
                                  double* __restrict__ out, const double* __restrict__ add) {
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (w >= nv) return;
  double t = 0.0;
  for (int bk = lane; bk < nblk; bk += 32) t += partial[bk * kMaxV + w];
  t = warp_sum(t);
  if (lane == 0) out[w] = t + (add ? add[w] : 0.0);
}

// r = b - r (in place on r)
__global__ void __launch_bounds__(256) k_residual(long long n, const double* __restrict__ b,
                                                  double* __restrict__ r) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    r[t] = b[t] - r[t];
}

// x += dinv .* sum_i y_i V_i  (nv from *d_nv when given)
__global__ void __launch_bounds__(256) k_combine(long long n, const double* __restrict__ V,
                                                 const double* __restrict__ y, int nv,
                                                 const int* __restrict__ d_nv,
                                                 const double* __restrict__ dinv,
                                                 double* __restrict__ x) {
  __shared__ double s_y[kMaxV];
  if (d_nv) nv = *d_nv;
  if (threadIdx.x < kMaxV) s_y[threadIdx.x] = threadIdx.x < nv ? y[threadIdx.x] : 0.0;
  __syncthreads();
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    double a = 0.0;
    for (int i = 0; i < nv; i++) a += s_y[i] * V[(size_t)i * n + t];
    x[t] += (dinv ? dinv[t] : 1.0) * a;
  }
}

// partial norms of one vector
__global__ void __launch_bounds__(256) k_norm2(long long n, const double* __restrict__ v,
                                               double* __restrict__ partial) {
  double acc[1] = {0.0};
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    acc[0] += v[t] * v[t];
  block_store_partials<1>(acc, 1, partial);
}

// GMRES least-squares state on the device: the Hessenberg columns after the
// Givens rotations (row stride kMaxV), the rotations, the rotated right-hand
// side g (|g[j]| = residual norm after j steps), the solution y, and the
// step count jj / converged flag that the host polls.
struct GmState {
  double H[(kMaxV + 1) * kMaxV];
  double cs[kMaxV], sn[kMaxV];
  double g[kMaxV + 1];
  double y[kMaxV];
  double target;
  int jj;    // columns processed in this cycle
  int done;  // |g[jj]| <= target, or breakdown
  double bn2, rn2;  // graph cycle (k_gm_first, k_gm_status): ||b||^2, end-of-cycle ||r||^2
};
static_assert(kGmOffset * sizeof(double) + sizeof(GmState) <= 12288 * sizeof(double),
              "GmState must fit in d_red");
static_assert(kRedBlocks * kMaxV + 2 * kMaxV + 8 + kMaxV <= kGmOffset, "d_red layout");

// start of a cycle: g = (||r||, 0, ...); *n2 = ||r||^2
__global__ void k_gm_start(GmState* __restrict__ S, const double* __restrict__ n2, double target) {
  if (threadIdx.x != 0) return;
  for (int i = 0; i <= kMaxV; i++) S->g[i] = 0.0;
  S->g[0] = sqrt(*n2);
  S->target = target;
  S->jj = 0;
  S->done = 0;
}

// start of the first cycle from x0 = 0 (r = b): g = (||b||, 0, ...), target
// tol ||b|| on the device; keeps ||b||^2 for the host's single read
__global__ void k_gm_first(GmState* __restrict__ S, const double* __restrict__ n2, double tol) {
  if (threadIdx.x != 0) return;
  for (int i = 0; i <= kMaxV; i++) S->g[i] = 0.0;
  const double b2 = *n2;
  S->g[0] = sqrt(b2);
  S->target = tol * sqrt(b2);
  S->jj = 0;
  S->done = 0;
  S->bn2 = b2;
  S->rn2 = -1.0;
}

// end of the graph cycle: the true residual's ||r||^2 next to jj, done, ||b||^2
__global__ void k_gm_status(GmState* __restrict__ S, const double* __restrict__ n2) {
  if (threadIdx.x == 0) S->rn2 = *n2;
}

// Arnoldi column jj: h = h1 + h2 (the two CGS passes), h[jj+1] = ||w||; apply
// the previous rotations, form rotation jj, update g.  Frozen once done, so
// steps launched past convergence change nothing the solution uses.  One thread.
__device__ void gm_update(GmState* __restrict__ S, int jj, const double* h1, const double* h2,
                          double n2) {
  if (S->done) return;
  double* H = S->H;
  for (int i = 0; i <= jj; i++) H[i * kMaxV + jj] = h1[i] + h2[i];
  const double hn = sqrt(n2);
  H[(jj + 1) * kMaxV + jj] = hn;
  for (int i = 0; i < jj; i++) {
    const double a = H[i * kMaxV + jj], b = H[(i + 1) * kMaxV + jj];
    H[i * kMaxV + jj] = S->cs[i] * a + S->sn[i] * b;
    H[(i + 1) * kMaxV + jj] = -S->sn[i] * a + S->cs[i] * b;
  }
  const double a = H[jj * kMaxV + jj], b = H[(jj + 1) * kMaxV + jj];
  const double r = sqrt(a * a + b * b);
  const double c = r > 0.0 ? a / r : 1.0, s = r > 0.0 ? b / r : 0.0;
  S->cs[jj] = c;
  S->sn[jj] = s;
  H[jj * kMaxV + jj] = r;
  H[(jj + 1) * kMaxV + jj] = 0.0;
  S->g[jj + 1] = -s * S->g[jj];
  S->g[jj] = c * S->g[jj];
  S->jj = jj + 1;
  if (fabs(S->g[jj + 1]) <= S->target || hn == 0.0) S->done = 1;
}

// y = R^-1 g on the processed columns (back substitution)
__global__ void k_gm_solve(GmState* __restrict__ S) {
  if (threadIdx.x != 0) return;
  const int j = S->jj;
  for (int i = j - 1; i >= 0; i--) {
    double t = S->g[i];
    for (int q = i + 1; q < j; q++) t -= S->H[i * kMaxV + q] * S->y[q];
    const double d = S->H[i * kMaxV + i];
    S->y[i] = d != 0.0 ? t / d : 0.0;
  }
}

// one CGS2 Arnoldi orthogonalisation with a register budget fitted to nv
// ---- Krylov vectors in FP32 pairs ----------------------------------------------
// One whole Arnoldi step after the operator runs in one cooperative launch
// (co-resident CTAs, grid-wide barriers between the phases): CGS2 against
// V_0..V_nv-1 (h1 = V^T w, w -= V h1, h2 = V^T w, w -= V h2), ||w||,
// V_nv = w / ||w||, and the Givens update of the least-squares state.  Every
// CTA reduces the per-CTA partial sums of a phase itself, so the phases need
// no further launches; each phase writes its own partial buffer.
constexpr int kArnThreads = 256;
// The Arnoldi basis and the operator output are stored as FP32 pairs (hi, lo:
// 48 significant bits, the bytes of a double vector): FP64 arithmetic runs at
// ~1/70 of the FP32 rate on this part, and CGS2 is 4 nv n multiply-adds per
// step, so the sweeps run in pair arithmetic and only per-block sums touch FP64.

// a += (xh + xl)(yh + yl)
__device__ __forceinline__ void ff_dot_acc(FF& a, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  ff_acc(a, p, fmaf(xh, yl, fmaf(xl, yh, fmaf(xh, yh, -p))));
}
__device__ __forceinline__ FF ff_shfl_xor(const FF& a, int o) {
  return FF{__shfl_xor_sync(0xffffffffu, a.s, o), __shfl_xor_sync(0xffffffffu, a.q, o)};
}
__device__ __forceinline__ FF ff_warp_sum(FF a) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const FF b = ff_shfl_xor(a, o);
    ff_acc(a, b.s, b.q);
  }
  return a;
}

// Reduce acc[0..nv) over the block into row[2i], row[2i+1] (a pair per entry).
template <int NVM>
__device__ __forceinline__ void arn_block_store_ff(const FF (&acc)[NVM], int nv, float* __restrict__ row,
                                                   float* __restrict__ s_red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NVM; i++) {
    if (i < nv) {
      const FF v = ff_warp_sum(acc[i]);
      if (lane == 0) {
        s_red[2 * (wid * kMaxV + i)] = v.s;
        s_red[2 * (wid * kMaxV + i) + 1] = v.q;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    FF t{0.f, 0.f};
    for (int w = 0; w < kArnThreads / 32; w++)
      ff_acc(t, s_red[2 * (w * kMaxV + threadIdx.x)], s_red[2 * (w * kMaxV + threadIdx.x) + 1]);
    t = ff_norm(t);
    row[2 * threadIdx.x] = t.s;
    row[2 * threadIdx.x + 1] = t.q;
  }
  __syncthreads();
}

// Sum of the blocks' pairs: s_out[i] (FP64) and s_outf[i] (the pair, renormalised)
__device__ __forceinline__ void arn_grid_reduce_ff(const float* __restrict__ part, int nblk, int nv,
                                                   double* __restrict__ s_out, float (*s_outf)[2]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int i = wid; i < nv; i += kArnThreads / 32) {
    FF t{0.f, 0.f};
    for (int b = lane; b < nblk; b += 32)
      ff_acc(t, __ldcg(part + 2 * ((size_t)b * kMaxV + i)), __ldcg(part + 2 * ((size_t)b * kMaxV + i) + 1));
    t = ff_norm(ff_warp_sum(t));
    if (lane == 0) {
      s_out[i] = (double)t.s + (double)t.q;
      s_outf[i][0] = t.s;
      s_outf[i][1] = t.q;
    }
  }
  __syncthreads();
}

// One Arnoldi step on pair vectors: CGS2 of w against V_0..V_{nv-1},
// V_nv = w / ||w||, and the Givens update of the least-squares state.  The
// sweeps are latency-bound at the occupancy the accumulators allow, so each
// thread moves L consecutive elements per load (L = 4: 16-byte loads of every
// hi and lo stream, when n is a multiple of 4; else L = 1).
template <int L>
__device__ __forceinline__ void ldv(const float* __restrict__ p, long long t, float (&o)[L]) {
  if constexpr (L == 4) {
    const float4 q = reinterpret_cast<const float4*>(p)[t];
    o[0] = q.x; o[1] = q.y; o[2] = q.z; o[3] = q.w;
  } else if constexpr (L == 2) {
    const float2 q = reinterpret_cast<const float2*>(p)[t];
    o[0] = q.x; o[1] = q.y;
  } else {
    o[0] = p[t];
  }
}
template <int L>
__device__ __forceinline__ void stv(float* __restrict__ p, long long t, const float (&o)[L]) {
  if constexpr (L == 4) {
    reinterpret_cast<float4*>(p)[t] = make_float4(o[0], o[1], o[2], o[3]);
  } else if constexpr (L == 2) {
    reinterpret_cast<float2*>(p)[t] = make_float2(o[0], o[1]);
  } else {
    p[t] = o[0];
  }
}

template <int NVM, int L>
__global__ void __launch_bounds__(kArnThreads) k_arnoldi_ff(long long n, const float* __restrict__ V,
                                                             float* __restrict__ w, int nv,
                                                             float* __restrict__ vnext,
                                                             float* __restrict__ part, GmState* gs,
                                                             int jj, float* __restrict__ xf,
                                                             const float* __restrict__ dh) {
  cg::grid_group grid = cg::this_grid();
  __shared__ float s_red[2 * (kArnThreads / 32) * kMaxV];
  __shared__ double s_h1[kMaxV], s_h2[kMaxV], s_n2[1];
  __shared__ float s_f1[kMaxV][2], s_f2[kMaxV][2], s_fn[1][2];
  const int nblk = gridDim.x;
  float* pA = part;
  float* pB = part + 2 * (size_t)nblk * kMaxV;
  float* pC = pB + 2 * (size_t)nblk * kMaxV;
  const long long nl = n / L;
  const long long stride = (long long)nblk * kArnThreads;
  const long long t0 = (long long)blockIdx.x * kArnThreads + threadIdx.x;
  float* wl = w + n;
  auto vh = [&](int i) { return V + 2 * (size_t)i * n; };
  FF acc[NVM];
  // pass 1: h1 = V^T w
#pragma unroll
  for (int i = 0; i < NVM; i++) acc[i] = FF{0.f, 0.f};
  for (long long t = t0; t < nl; t += stride) {
    float a[L], b[L];
    ldv<L>(w, t, a);
    ldv<L>(wl, t, b);
#pragma unroll
    for (int i = 0; i < NVM; i++)
      if (i < nv) {
        float x[L], y[L];
        ldv<L>(vh(i), t, x);
        ldv<L>(vh(i) + n, t, y);
#pragma unroll
        for (int k = 0; k < L; k++) ff_dot_acc(acc[i], x[k], y[k], a[k], b[k]);
      }
  }
  arn_block_store_ff<NVM>(acc, nv, pA + 2 * (size_t)blockIdx.x * kMaxV, s_red);
  grid.sync();
  arn_grid_reduce_ff(pA, nblk, nv, s_h1, s_f1);
  // pass 2: w -= V h1; h2 = V^T w
#pragma unroll
  for (int i = 0; i < NVM; i++) acc[i] = FF{0.f, 0.f};
  for (long long t = t0; t < nl; t += stride) {
    float a[L], b[L];
    ldv<L>(w, t, a);
    ldv<L>(wl, t, b);
    FF wt[L];
#pragma unroll
    for (int k = 0; k < L; k++) wt[k] = FF{a[k], b[k]};
#pragma unroll
    for (int i = 0; i < NVM; i++)
      if (i < nv) {
        float x[L], y[L];
        ldv<L>(vh(i), t, x);
        ldv<L>(vh(i) + n, t, y);
#pragma unroll
        for (int k = 0; k < L; k++) {
          const FF u = ff_mul(x[k], y[k], s_f1[i][0], s_f1[i][1]);
          ff_acc(wt[k], -u.s, -u.q);
        }
      }
#pragma unroll
    for (int k = 0; k < L; k++) {
      wt[k] = ff_norm(wt[k]);
      a[k] = wt[k].s;
      b[k] = wt[k].q;
    }
    stv<L>(w, t, a);
    stv<L>(wl, t, b);
    // the V loads again (cache hits) rather than 2 L more registers per vector
#pragma unroll
    for (int i = 0; i < NVM; i++)
      if (i < nv) {
        float x[L], y[L];
        ldv<L>(vh(i), t, x);
        ldv<L>(vh(i) + n, t, y);
#pragma unroll
        for (int k = 0; k < L; k++) ff_dot_acc(acc[i], x[k], y[k], a[k], b[k]);
      }
  }
  arn_block_store_ff<NVM>(acc, nv, pB + 2 * (size_t)blockIdx.x * kMaxV, s_red);
  grid.sync();
  arn_grid_reduce_ff(pB, nblk, nv, s_h2, s_f2);
  // pass 3: w -= V h2; ||w||^2
  FF nacc[1] = {FF{0.f, 0.f}};
  for (long long t = t0; t < nl; t += stride) {
    float a[L], b[L];
    ldv<L>(w, t, a);
    ldv<L>(wl, t, b);
    FF wt[L];
#pragma unroll
    for (int k = 0; k < L; k++) wt[k] = FF{a[k], b[k]};
#pragma unroll
    for (int i = 0; i < NVM; i++)
      if (i < nv) {
        float x[L], y[L];
        ldv<L>(vh(i), t, x);
        ldv<L>(vh(i) + n, t, y);
#pragma unroll
        for (int k = 0; k < L; k++) {
          const FF u = ff_mul(x[k], y[k], s_f2[i][0], s_f2[i][1]);
          ff_acc(wt[k], -u.s, -u.q);
        }
      }
#pragma unroll
    for (int k = 0; k < L; k++) {
      wt[k] = ff_norm(wt[k]);
      a[k] = wt[k].s;
      b[k] = wt[k].q;
      ff_dot_acc(nacc[0], a[k], b[k], a[k], b[k]);
    }
    stv<L>(w, t, a);
    stv<L>(wl, t, b);
  }
  arn_block_store_ff<1>(nacc, 1, pC + 2 * (size_t)blockIdx.x * kMaxV, s_red);
  grid.sync();
  arn_grid_reduce_ff(pC, nblk, 1, s_n2, s_fn);
  // V_nv = w / ||w|| (the elements this thread wrote in pass 3)
  const double inv = s_n2[0] > 0.0 ? 1.0 / sqrt(s_n2[0]) : 0.0;
  const float ih = (float)inv, il = (float)(inv - (double)ih);
  for (long long t = t0; t < nl; t += stride) {
    float a[L], b[L];
    ldv<L>(w, t, a);
    ldv<L>(wl, t, b);
#pragma unroll
    for (int k = 0; k < L; k++) {
      const FF u = ff_norm(ff_mul(a[k], b[k], ih, il));
      a[k] = u.s;
      b[k] = u.q;
    }
    stv<L>(vnext, t, a);
    stv<L>(vnext + n, t, b);
    if (xf) {
      // the next operator's FP32 input fp32(D V_nv), written while it is in registers
      if (dh) {
        float dd[L];
        ldv<L>(dh, t, dd);
#pragma unroll
        for (int k = 0; k < L; k++) a[k] *= dd[k];
      }
      stv<L>(xf, t, a);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) gm_update(gs, jj, s_h1, s_h2, s_n2[0]);
}

template <int NVM, int L>
cudaError_t launch_arnoldi_ff_l(cudaStream_t s, long long n, const float* V, float* w, int nv,
                                float* vnext, float* part, GmState* gs, int jj, float* xf, const float* dh) {
  static int grid[64] = {0};  // per device: co-resident CTAs
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  if (grid[dev] == 0) {
    int sms = 0, per = 0;
    cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_arnoldi_ff<NVM, L>, kArnThreads, 0);
    if (e != cudaSuccess) return e;
    if (per < 1) return cudaErrorLaunchOutOfResources;
    grid[dev] = std::min(sms * per, kArnMaxGrid);
  }
  const long long want = (n / L + kArnThreads - 1) / kArnThreads;
  const unsigned g = (unsigned)std::max<long long>(1, std::min<long long>(grid[dev], want));
  void* args[] = {&n, &V, &w, &nv, &vnext, &part, &gs, &jj, &xf, &dh};
  return cudaLaunchCooperativeKernel((const void*)k_arnoldi_ff<NVM, L>, dim3(g), dim3(kArnThreads), args, 0, s);
}

// the widest streams at which every pair vector's hi and lo start aligned
template <int NVM>
cudaError_t launch_arnoldi_ff(cudaStream_t s, long long n, const float* V, float* w, int nv,
                              float* vnext, float* part, GmState* gs, int jj, float* xf, const float* dh) {
  if (n % 4 == 0) return launch_arnoldi_ff_l<NVM, 4>(s, n, V, w, nv, vnext, part, gs, jj, xf, dh);
  if (n % 2 == 0) return launch_arnoldi_ff_l<NVM, 2>(s, n, V, w, nv, vnext, part, gs, jj, xf, dh);
  return launch_arnoldi_ff_l<NVM, 1>(s, n, V, w, nv, vnext, part, gs, jj, xf, dh);
}

// V0 = r / ||r|| as a pair vector (nrm2: ||r||^2)
__global__ void __launch_bounds__(256) k_start_ff(long long n, const double* __restrict__ r,
                                                  const double* __restrict__ nrm2, float* __restrict__ v,
                                                  float* __restrict__ xf, const float* __restrict__ dh) {
  const double sc = *nrm2 > 0.0 ? 1.0 / sqrt(*nrm2) : 0.0;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const double x = r[t] * sc;
    const float h = (float)x;
    v[t] = h;
    v[n + t] = (float)(x - (double)h);
    if (xf) xf[t] = dh ? h * dh[t] : h;  // the first operator's FP32 input
  }
}

// double vector <-> pair vector
__global__ void __launch_bounds__(256) k_to_ff(long long n, const double* __restrict__ x, float* __restrict__ v) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const double a = x[t];
    const float h = (float)a;
    v[t] = h;
    v[n + t] = (float)(a - (double)h);
  }
}
__global__ void __launch_bounds__(256) k_from_ff(long long n, const float* __restrict__ v, double* __restrict__ x) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    x[t] = (double)v[t] + (double)v[n + t];
}

// x += D sum_i y_i V_i, V pair vectors, D as pairs (or none); nv from *d_nv
// (at most NVM: the loads of all vectors are issued before the pair sums)
template <int NVM>
__global__ void __launch_bounds__(256) k_combine_ff(long long n, const float* __restrict__ V,
                                                    const double* __restrict__ y,
                                                    const int* __restrict__ d_nv,
                                                    const float* __restrict__ dff,
                                                    double* __restrict__ x) {
  __shared__ float s_y[kMaxV][2];
  const int nv = min(*d_nv, NVM);
  if (threadIdx.x < kMaxV) {
    const double v = threadIdx.x < nv ? y[threadIdx.x] : 0.0;
    s_y[threadIdx.x][0] = (float)v;
    s_y[threadIdx.x][1] = (float)(v - (double)s_y[threadIdx.x][0]);
  }
  __syncthreads();
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    float vh[NVM], vl[NVM];
#pragma unroll
    for (int i = 0; i < NVM; i++)
      if (i < nv) {
        vh[i] = V[2 * (size_t)i * n + t];
        vl[i] = V[2 * (size_t)i * n + n + t];
      }
    FF a{0.f, 0.f};
#pragma unroll
    for (int i = 0; i < NVM; i++)
      if (i < nv) {
        const FF u = ff_mul(vh[i], vl[i], s_y[i][0], s_y[i][1]);
        ff_acc(a, u.s, u.q);
      }
    a = ff_norm(a);
    if (dff) a = ff_mul(a.s, a.q, dff[t], dff[n + t]);
    x[t] += ff_value(a);
  }
}

void launch_combine_ff(cudaStream_t s, unsigned gr, long long n, const float* V, const double* y,
                       const int* d_nv, int nv_host, const float* dff, double* x) {
  if (nv_host <= 4)
    k_combine_ff<4><<<gr, 256, 0, s>>>(n, V, y, d_nv, dff, x);
  else if (nv_host <= 8)
    k_combine_ff<8><<<gr, 256, 0, s>>>(n, V, y, d_nv, dff, x);
  else if (nv_host <= 16)
    k_combine_ff<16><<<gr, 256, 0, s>>>(n, V, y, d_nv, dff, x);
  else
    k_combine_ff<32><<<gr, 256, 0, s>>>(n, V, y, d_nv, dff, x);
}

// the Jacobi scaling D as pairs
__global__ void __launch_bounds__(256) k_dff(long long n, const double* __restrict__ d, float* __restrict__ v) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const float h = (float)d[t];
    v[t] = h;
    v[n + t] = (float)(d[t] - (double)h);
  }
}

// xf = fp32(D v)
__global__ void __launch_bounds__(256) k_in_f32(long long n, OpIn in, float* __restrict__ xf) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    xf[t] = in.vd ? (float)in.vd[t] : (in.dh ? in.vh[t] * in.dh[t] : in.vh[t]);
}

// w = A (D v) with the identity part in pairs and the rest in FP32 (the FP32
// inner operator of k_matvec32 with pair input and output)
__global__ void __launch_bounds__(256) k_matvec32_ff(long long ncor, const int* __restrict__ nbr,
                                                     const float* __restrict__ M,
                                                     const float* __restrict__ xf, OpIn in,
                                                     float* __restrict__ wh, float* __restrict__ wl,
                                                     TapsF T) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * ncor) return;
  const int p = (int)(t / ncor);
  const long long c = t - (long long)p * ncor;
  int b, i, j, k;
  corner_ijk(c, b, i, j, k);
  float acc = 0.f;
#pragma unroll 3
  for (int s = 0; s < 27; s++) {
    const int dig[3] = {s % 3, (s / 3) % 3, s / 9};
    const int di = dig[0] == 0 ? 0 : (dig[0] == 1 ? -1 : 1);
    const int dj = dig[1] == 0 ? 0 : (dig[1] == 1 ? -1 : 1);
    const int dk = dig[2] == 0 ? 0 : (dig[2] == 1 ? -1 : 1);
    const int nb = local_id(nbr, b, i + di, j + dj, k + dk);
    const float* Ms = M + (size_t)(9 * s + 3 * p) * ncor + c;
#pragma unroll
    for (int q = 0; q < 3; q++)
      acc = fmaf(fmaf(T.f, Ms[(size_t)q * ncor], T.K[p][q][s]), xf[q * ncor + nb], acc);
  }
  FF y = opin_value(in, t);
  ff_acc(y, acc, 0.f);
  y = ff_norm(y);
  wh[t] = y.s;
  wl[t] = y.q;
}

// ---- field updates -----------------------------------------------------------
__global__ void __launch_bounds__(256) k_update_b(long long ncor, const int* __restrict__ nbr,
                                                  const double* __restrict__ Eh,
                                                  const double* __restrict__ Bn,
                                                  double* __restrict__ Bnew, double c4x,
                                                  double c4y, double c4z) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncor) return;
  int b, i, j, k;
  corner_ijk(c, b, i, j, k);
  double Ex[2][2][2], Ey[2][2][2], Ez[2][2][2];
#pragma unroll
  for (int kk = 0; kk < 2; kk++)
#pragma unroll
    for (int jj = 0; jj < 2; jj++)
#pragma unroll
      for (int ii = 0; ii < 2; ii++) {
        const int id = local_id(nbr, b, i + ii, j + jj, k + kk);
        Ex[ii][jj][kk] = Eh[id];
        Ey[ii][jj][kk] = Eh[ncor + id];
        Ez[ii][jj][kk] = Eh[2 * ncor + id];
      }
  double t0 = 0.0, t1 = 0.0, t2 = 0.0;
#pragma unroll
  for (int ii = 0; ii < 2; ii++)
#pragma unroll
    for (int jj = 0; jj < 2; jj++) {
      t0 += -c4y * (Ez[ii][1][jj] - Ez[ii][0][jj]) + c4z * (Ey[ii][jj][1] - Ey[ii][jj][0]);
      t1 += -c4z * (Ex[ii][jj][1] - Ex[ii][jj][0]) + c4x * (Ez[1][ii][jj] - Ez[0][ii][jj]);
      t2 += -c4x * (Ey[1][ii][jj] - Ey[0][ii][jj]) + c4y * (Ex[ii][1][jj] - Ex[ii][0][jj]);
    }
  Bnew[c] = Bn[c] + t0;
  Bnew[ncor + c] = Bn[ncor + c] + t1;
  Bnew[2 * ncor + c] = Bn[2 * ncor + c] + t2;
}

__global__ void __launch_bounds__(256) k_c2n(long long ncor, const int* __restrict__ nbr,
                                             const double* __restrict__ Bc,
                                             double* __restrict__ Bcor) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncor) return;
  int b, i, j, k;
  corner_ijk(c, b, i, j, k);
  double t[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int kk = -1; kk <= 0; kk++)
#pragma unroll
    for (int jj = -1; jj <= 0; jj++)
#pragma unroll
      for (int ii = -1; ii <= 0; ii++) {
        const int id = local_id(nbr, b, i + ii, j + jj, k + kk);
#pragma unroll
        for (int d = 0; d < 3; d++) t[d] += Bc[d * ncor + id];
      }
#pragma unroll
  for (int d = 0; d < 3; d++) Bcor[d * ncor + c] = t[d] / 8.0;
}

__global__ void __launch_bounds__(256) k_update_e(long long ncor, const double* __restrict__ Eh,
                                                  double* __restrict__ En,
                                                  const double* __restrict__ Bc, double theta,
                                                  double vol_over_8pi, double* __restrict__ energy) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double en = 0.0;
  if (c < ncor) {
    double e2 = 0.0, b2 = 0.0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double e = (Eh[d * ncor + c] - (1.0 - theta) * En[d * ncor + c]) / theta;
      En[d * ncor + c] = e;
      e2 += e * e;
      const double bb = Bc[d * ncor + c];
      b2 += bb * bb;
    }
    en = (e2 + b2) * vol_over_8pi;
  }
  __shared__ double s[8];
  en = warp_sum(en);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = en;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s[w];
    atomicAdd(energy, t);
  }
}

__global__ void __launch_bounds__(256) k_add(long long n, const double* __restrict__ a,
                                             const double* __restrict__ b, double* __restrict__ o) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    o[t] = a[t] + b[t];
}

unsigned grid1(long long n) { return (unsigned)((n + 255) / 256); }
unsigned gridt(long long n, int tb) { return (unsigned)((n + tb - 1) / tb); }
// sweep/reduction grid: at least ept elements per thread, at most cap CTAs
unsigned gridr(long long n, int cap = kRedBlocks, int ept = 4) {
  long long g = (n + 256LL * ept - 1) / (256LL * ept);
  if (g > cap) g = cap;
  return (unsigned)(g < 1 ? 1 : g);
}

}  // namespace

// ============================================================================
// FP32 pair split of an operator input into the context's scratch (hi_only:
// the FP32 rounding alone).  d_xs is also where k_start_ff / k_arnoldi_ff
// leave the FP32 input of the next Krylov vector's operator application: this
// split, k_rhs and the AMR operators overwrite it, so none of them may run
// between an Arnoldi step and the operator application that follows it.
static cudaError_t split_input(amps_gpu_ctx* c, const double* x, const double* dinv,
                               bool hi_only = false) {
  const long long n = 3 * c->nvc;
  if (!c->d_xs) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&c->d_xs), sizeof(float) * 2 * n);
    if (e != cudaSuccess) return e;
  }
  k_split<<<gridr(n), 256, 0, c->stream>>>(n, x, dinv, c->d_xs, hi_only ? nullptr : c->d_xs + n);
  return cudaGetLastError();
}

cudaError_t launch_matvec(amps_gpu_ctx* c, const double* x, const double* dinv, double* y) {
  if (c->amr) return launch_amr_matvec(c, x, dinv, y);
  const TapsFF T = taps_ff(make_taps(c->cfg, true));
  TimedLaunch t(c, "matvec", 2);
  cudaError_t e = split_input(c, x, dinv);
  if (e != cudaSuccess) return e;
  const long long n = 3 * c->ncor;
  k_matvec<<<gridt(n, c->tune_tb), c->tune_tb, 0, c->stream>>>(c->ncor, c->d_nbr, c->d_M,
                                                               c->d_xs, c->d_xs + n, y, T);
  return cudaGetLastError();
}

cudaError_t launch_matvec32(amps_gpu_ctx* c, const double* x, const double* dinv, double* y) {
  if (c->amr) return launch_amr_matvec32(c, x, dinv, y);
  const TapsF T = taps_f32(make_taps(c->cfg, false));
  TimedLaunch t(c, "matvec32", 2);
  cudaError_t e = split_input(c, x, dinv, true);
  if (e != cudaSuccess) return e;
  k_matvec32<<<gridt(3 * c->ncor, c->tune_tb), c->tune_tb, 0, c->stream>>>(c->ncor, c->d_nbr,
                                                                            c->d_M, c->d_xs, x, dinv, y, T);
  return cudaGetLastError();
}

cudaError_t launch_in_f32(amps_gpu_ctx* c, const OpIn& in, float* xf) {
  const long long n = 3 * c->nvc;
  k_in_f32<<<gridr(n), 256, 0, c->stream>>>(n, in, xf);
  return cudaGetLastError();
}

cudaError_t launch_matvec32_ff(amps_gpu_ctx* c, const OpIn& in, float* wh, float* wl) {
  if (c->amr) return launch_amr_matvec32_ff(c, in, wh, wl);
  const long long n = 3 * c->ncor;
  if (!c->d_xs) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&c->d_xs), sizeof(float) * 2 * n);
    if (e != cudaSuccess) return e;
  }
  const TapsF T = taps_f32(make_taps(c->cfg, false));
  TimedLaunch t(c, "matvec32", in.xf_ready ? 1 : 2);
  cudaError_t e = in.xf_ready ? cudaSuccess : launch_in_f32(c, in, c->d_xs);
  if (e != cudaSuccess) return e;
  k_matvec32_ff<<<gridt(n, c->tune_tb), c->tune_tb, 0, c->stream>>>(c->ncor, c->d_nbr, c->d_M, c->d_xs, in,
                                                                     wh, wl, T);
  return cudaGetLastError();
}

cudaError_t launch_rhs(amps_gpu_ctx* c) {
  if (c->amr) return launch_amr_rhs(c);
  const TapsFF T = taps_ff(make_taps(c->cfg, false));
  double c4[3];
  for (int d = 0; d < 3; d++) c4[d] = 0.25 * (c->cfg.dt / c->cfg.dx[d] * c->cfg.theta);
  TimedLaunch t(c, "rhs", 2);
  cudaError_t e = split_input(c, c->d_En, nullptr);
  if (e != cudaSuccess) return e;
  const long long n = 3 * c->ncor;
  k_rhs<<<grid1(n), 256, 0, c->stream>>>(c->ncor, c->d_nbr, c->d_M, c->d_xs, c->d_xs + n, c->d_Bc,
                                         c->d_J, c->d_rhs, T, c4[0], c4[1], c4[2]);
  return cudaGetLastError();
}

cudaError_t launch_jacobi_diag(amps_gpu_ctx* c) {
  if (c->amr) return launch_amr_jacobi(c);
  Taps T = make_taps(c->cfg, true);
  TimedLaunch t(c, "jacobi");
  k_jacobi<<<grid1(c->ncor), 256, 0, c->stream>>>(c->ncor, c->d_M, c->d_dinv, T.K[0][0][0],
                                                   T.K[1][1][0], T.K[2][2][0], T.f);
  return cudaGetLastError();
}

cudaError_t launch_update_b(amps_gpu_ctx* c) {
  if (c->amr) return launch_amr_update_b(c);
  double c4[3];
  for (int d = 0; d < 3; d++) c4[d] = 0.25 * (c->cfg.dt / c->cfg.dx[d]);
  TimedLaunch t(c, "update_b");
  k_update_b<<<grid1(c->ncor), 256, 0, c->stream>>>(c->ncor, c->d_nbr, c->d_Eh, c->d_Bc,
                                                     c->d_Bc2, c4[0], c4[1], c4[2]);
  return cudaGetLastError();
}

cudaError_t launch_c2n(amps_gpu_ctx* c, const double* Bcen, double* Bcor) {
  if (c->amr) return launch_amr_c2n(c, Bcen, Bcor);
  TimedLaunch t(c, "c2n");
  k_c2n<<<grid1(c->ncor), 256, 0, c->stream>>>(c->ncor, c->d_nbr, Bcen, Bcor);
  return cudaGetLastError();
}

cudaError_t launch_update_e(amps_gpu_ctx* c) {
  if (c->amr) return launch_amr_update_e(c);
  const double vol = c->cfg.dx[0] * c->cfg.dx[1] * c->cfg.dx[2];
  cudaError_t e = cudaMemsetAsync(c->d_energy + 1, 0, sizeof(double), c->stream);
  if (e != cudaSuccess) return e;
  TimedLaunch t(c, "update_e");
  k_update_e<<<grid1(c->ncor), 256, 0, c->stream>>>(c->ncor, c->d_Eh, c->d_En, c->d_Bc,
                                                     c->cfg.theta, vol * 0.125 / kPi,
                                                     c->d_energy + 1);
  return cudaGetLastError();
}

// GMRES(m) with right preconditioning, CGS2 Arnoldi, Givens rotations on the
// device, and iterative refinement across restarts: every cycle starts from
// the true FP64 residual r = b - A x, its Arnoldi steps apply the operator with
// its identity part in FP64 and the rest in FP32 (c->inner_fp32), and the solve
// ends when the FP64 residual satisfies ||b - A x|| <= tol ||b||.  The
// preconditioner is none (precond 0), Jacobi (1, z = D v) or the learned block
// network (2, z = D v + N(D v); flexible form: the directions z_j are kept).
// Each Arnoldi step is the operator plus one cooperative kernel (k_arnoldi:
// CGS2, normalisation and the Givens update).  The host does not wait for each
// step: it queues as many Arnoldi steps as the last cycle took before it first
// reads the device's convergence flag, then one step per read; steps queued
// past convergence leave the least-squares state untouched (gm_update is
// frozen), so they cost time but not accuracy.
// Device scratch layout of d_red: [0, kRedBlocks*kMaxV) partials, then h1
// (kMaxV), h2 (kMaxV), nrm2 (8), y (kMaxV); GmState at kGmOffset.
amps_gpu_status gmres_solve(amps_gpu_ctx* c, double tol, int maxit, int precond,
                            amps_gpu_solve_stats* st) {
  const long long n = 3 * c->nvc;
  const int m = std::min(c->restart, kMaxV);
  double* partial = c->d_red;
  double* d_n2 = c->d_red + kRedBlocks * kMaxV + 2 * kMaxV;
  GmState* gs = reinterpret_cast<GmState*>(c->d_red + kGmOffset);
  const unsigned gr = gridr(n, c->tune_red, c->tune_ept);
  cudaStream_t s = c->stream;
  cudaError_t e;
#define CK(x)                                                   \
  do {                                                          \
    e = (x);                                                    \
    if (e != cudaSuccess) return cuda_check(c, e, #x);          \
  } while (0)

  if (!c->d_arn)
    CK(cudaMalloc(reinterpret_cast<void**>(&c->d_arn), sizeof(double) * 3 * kArnMaxGrid * kMaxV));
  const double* dinv = precond >= 1 ? c->d_dinv : nullptr;
  const bool flexible = precond == 2;
  if (flexible && !c->d_Z)
    return set_err(c, AMPS_GPU_INVALID_ARG, "learned preconditioner: no network loaded");
  // Krylov vectors V_j and the operator output w are FP32 pair vectors (the
  // bytes of d_V / d_w); the Jacobi scaling is used as pairs
  float* Vf = reinterpret_cast<float*>(c->d_V);
  float* wf = reinterpret_cast<float*>(c->d_w);
  auto vf = [&](int j) { return Vf + 2 * (size_t)j * n; };
  const float* dh = nullptr;
  const float* dl = nullptr;
  if (dinv) {
    if (!c->d_dff) CK(cudaMalloc(reinterpret_cast<void**>(&c->d_dff), sizeof(float) * 2 * n));
    dh = c->d_dff;
    dl = c->d_dff + n;
  }
  const bool harvest = precond == 1 && c->pn;
  if ((flexible || harvest || !c->inner_fp32) && !c->d_tmpv)
    CK(cudaMalloc(reinterpret_cast<void**>(&c->d_tmpv), sizeof(double) * 2 * n));
  // w = A (D v_j), or A z_j for the flexible directions, as pairs
  // the FP32 operator input of the next Krylov vector is written by the step
  // that makes the vector (k_start_ff, k_arnoldi_ff) when the operator takes V
  // directly (no learned directions, FP32 inner operator)
  // (nothing that writes d_xs -- split_input, k_rhs, the AMR operators -- runs
  // between a step that writes it and the inner_matvec that reads it)
  const bool pre_xf = !flexible && c->inner_fp32;
  if (pre_xf && !c->d_xs) CK(cudaMalloc(reinterpret_cast<void**>(&c->d_xs), sizeof(float) * 2 * n));
  float* xf_next = pre_xf ? c->d_xs : nullptr;
  auto inner_matvec = [&](int jj, const double* zj) -> cudaError_t {
    if (c->inner_fp32) {
      OpIn in{};
      if (zj) {
        in.vd = zj;
      } else {
        in.vh = vf(jj);
        in.vl = vf(jj) + n;
        in.dh = dh;
        in.dl = dl;
        in.xf_ready = pre_xf;
      }
      return launch_matvec32_ff(c, in, wf, wf + n);
    }
    // FP64 inner operator, through FP64 copies
    const double* x = zj;
    if (!zj) {
      k_from_ff<<<gr, 256, 0, s>>>(n, vf(jj), c->d_tmpv);
      x = c->d_tmpv;
    }
    cudaError_t ee = launch_matvec(c, x, zj ? nullptr : dinv, c->d_tmpv + n);
    if (ee != cudaSuccess) return ee;
    k_to_ff<<<gr, 256, 0, s>>>(n, c->d_tmpv + n, wf);
    return cudaGetLastError();
  };
  auto norm_to = [&](const double* v) {
    k_norm2<<<gr, 256, 0, s>>>(n, v, partial);
    k_reduce_partials<<<1, 32, 0, s>>>(partial, gr, 1, d_n2, nullptr);
  };
  auto read_norm = [&](const double* v, double* out) -> cudaError_t {
    norm_to(v);
    cudaError_t ee = cudaMemcpyAsync(c->h_red, d_n2, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (ee != cudaSuccess) return ee;
    ee = cudaStreamSynchronize(s);
    *out = std::sqrt(c->h_red[0]);
    return ee;
  };
  // the Jacobi scaling, x0 = 0, r0 = b
  auto prologue = [&]() -> cudaError_t {
    if (dinv) {
      cudaError_t ee = launch_jacobi_diag(c);
      if (ee != cudaSuccess) return ee;
      k_dff<<<gr, 256, 0, s>>>(n, dinv, c->d_dff);
    }
    cudaError_t ee = cudaMemsetAsync(c->d_x, 0, sizeof(double) * n, s);
    if (ee == cudaSuccess)
      ee = cudaMemcpyAsync(c->d_w, c->d_rhs, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
    return ee;
  };
  // Arnoldi step jj: the operator (after the network for flexible directions),
  // then the cooperative CGS2 + normalisation + Givens step
  auto arnoldi_step = [&](int jj) -> cudaError_t {
    const int nv = jj + 1;
    cudaError_t ee;
    if (flexible) {
      double* zj = c->d_Z + (size_t)jj * n;
      k_from_ff<<<gr, 256, 0, s>>>(n, vf(jj), c->d_tmpv);  // v_j in FP64 for the network
      if ((ee = launch_precond_net(c, c->d_tmpv, zj)) != cudaSuccess) return ee;
      if ((ee = inner_matvec(jj, zj)) != cudaSuccess) return ee;
    } else {
      if ((ee = inner_matvec(jj, nullptr)) != cudaSuccess) return ee;
      // training pairs for the learned preconditioner: (A D v_j, D v_j)
      if (harvest) {
        k_from_ff<<<gr, 256, 0, s>>>(n, wf, c->d_tmpv);
        k_from_ff<<<gr, 256, 0, s>>>(n, vf(jj), c->d_tmpv + n);
        if ((ee = precond_harvest_pairs(c, c->d_tmpv, c->d_tmpv + n, 1)) != cudaSuccess) return ee;
      }
    }
    TimedLaunch t(c, "gmres_orth");
    float* part = reinterpret_cast<float*>(c->d_arn);
    float* vnext = vf(nv);
    if (nv <= 4) return launch_arnoldi_ff<4>(s, n, Vf, wf, nv, vnext, part, gs, jj, xf_next, dh);
    if (nv <= 8) return launch_arnoldi_ff<8>(s, n, Vf, wf, nv, vnext, part, gs, jj, xf_next, dh);
    if (nv <= 16) return launch_arnoldi_ff<16>(s, n, Vf, wf, nv, vnext, part, gs, jj, xf_next, dh);
    return launch_arnoldi_ff<32>(s, n, Vf, wf, nv, vnext, part, gs, jj, xf_next, dh);
  };
  // end of a cycle of at most nv_max steps: least squares, x += (D) V y, the
  // true FP64 residual into w and its squared norm into d_n2
  double* w = c->d_w;  // between cycles: the FP64 residual
  auto cycle_end = [&](int nv_max) -> cudaError_t {
    k_gm_solve<<<1, 32, 0, s>>>(gs);
    if (flexible)
      k_combine<<<gr, 256, 0, s>>>(n, c->d_Z, gs->y, kMaxV, &gs->jj, nullptr, c->d_x);
    else
      launch_combine_ff(s, gr, n, Vf, gs->y, &gs->jj, nv_max, dinv ? c->d_dff : nullptr, c->d_x);
    cudaError_t ee = cudaGetLastError();
    if (ee == cudaSuccess) ee = launch_matvec(c, c->d_x, nullptr, w);
    if (ee != cudaSuccess) return ee;
    k_residual<<<gr, 256, 0, s>>>(n, c->d_rhs, w);
    norm_to(w);
    return cudaGetLastError();
  };

  int it = 0, cycles = 0;
  bool conv = false;
  double rel = 0.0, bnorm = 0.0, beta = 0.0;
  // The first cycle as one CUDA graph when the previous solve with this
  // preconditioner tells how many Arnoldi steps to queue (K): prologue, ||b||
  // and the cycle start on the device, K steps, the cycle end, one read of
  // (steps used, converged, ||b||^2, ||r||^2).  Steps past convergence are
  // frozen; a cycle that needed more than K steps ends as a restart.  Later
  // cycles run as below.
  const int K = std::max(1, std::min({c->gm_guess[precond], m, maxit}));
  const bool graph = c->use_graphs && !c->timing && !flexible && !harvest && c->inner_fp32 &&
                     c->gm_guess[precond] > 0 && !c->solve_graphs_off;
  bool graph_done = false;
  if (graph) {
    cudaGraphExec_t exec = nullptr;
    for (auto& g : c->solve_graphs)
      if (g.precond == precond && g.steps == K && g.tb == c->tune_tb && g.red == c->tune_red &&
          g.ept == c->tune_ept)
        exec = g.exec;
    if (!exec) {
      cudaGraph_t gr_cap = nullptr;
      cudaError_t ee = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
      if (ee == cudaSuccess) {
        cudaError_t e1 = prologue();
        if (e1 == cudaSuccess) {
          norm_to(c->d_rhs);
          k_gm_first<<<1, 32, 0, s>>>(gs, d_n2, tol);
          k_start_ff<<<gr, 256, 0, s>>>(n, w, d_n2, vf(0), xf_next, dh);
          for (int jj = 0; jj < K && e1 == cudaSuccess; jj++) e1 = arnoldi_step(jj);
        }
        if (e1 == cudaSuccess) e1 = cycle_end(K);
        if (e1 == cudaSuccess) {
          k_gm_status<<<1, 32, 0, s>>>(gs, d_n2);
          e1 = cudaMemcpyAsync(c->h_red, &gs->jj, 2 * sizeof(int) + 2 * sizeof(double),
                               cudaMemcpyDeviceToHost, s);
        }
        ee = cudaStreamEndCapture(s, &gr_cap);
        if (ee == cudaSuccess && e1 == cudaSuccess)
          ee = cudaGraphInstantiate(&exec, gr_cap, 0);
        else if (ee == cudaSuccess)
          ee = e1;
        if (gr_cap) cudaGraphDestroy(gr_cap);
      }
      if (ee != cudaSuccess || !exec) {
        // not capturable here: clear the error state of the capture, solve eagerly
        cudaGetLastError();
        c->solve_graphs_off = true;
        exec = nullptr;
      } else {
        if (c->solve_graphs.size() >= 8) {
          cudaGraphExecDestroy(c->solve_graphs.front().exec);
          c->solve_graphs.erase(c->solve_graphs.begin());
        }
        c->solve_graphs.push_back({precond, K, c->tune_tb, c->tune_red, c->tune_ept, exec});
      }
    }
    if (exec) {
      CK(cudaGraphLaunch(exec, s));
      CK(cudaStreamSynchronize(s));
      const int* stat = reinterpret_cast<const int*>(c->h_red);
      it = stat[0];
      cycles = 1;
      bnorm = std::sqrt(c->h_red[1]);
      beta = std::sqrt(std::max(0.0, c->h_red[2]));
      graph_done = true;
    }
  }
  if (!graph_done) {
    CK(prologue());
    CK(read_norm(c->d_rhs, &bnorm));
    beta = bnorm;
  }
  while (true) {
    rel = bnorm > 0.0 ? beta / bnorm : 0.0;
    if (rel <= tol) {
      conv = true;
      break;
    }
    if (it >= maxit) break;
    cycles++;
    // the FP32 operators keep the identity part in FP64 accuracy (their noise
    // is ~1e-7 of the off-identity terms), so a cycle runs to the tolerance; a
    // later cycle only corrects what that noise left
    const double target = tol * bnorm;
    // V0 = r / ||r|| (d_n2 holds ||r||^2)
    k_gm_start<<<1, 32, 0, s>>>(gs, d_n2, target);
    k_start_ff<<<gr, 256, 0, s>>>(n, w, d_n2, vf(0), xf_next, dh);
    int launched = 0, used = 0;
    bool done = false;
    const int first_read = cycles == 1 ? std::max(1, std::min(c->gm_guess[precond], m)) : 1;
    while (!done && launched < m && it + launched < maxit) {
      CK(arnoldi_step(launched++));
      CK(cudaGetLastError());
      if (launched >= first_read || launched == m || it + launched >= maxit) {
        CK(cudaMemcpyAsync(c->h_red, &gs->jj, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        const int* stat = reinterpret_cast<const int*>(c->h_red);
        used = stat[0];
        done = stat[1] != 0;
      }
    }
    it += used;
    CK(cycle_end(used));
    CK(cudaMemcpyAsync(c->h_red, d_n2, sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    beta = std::sqrt(c->h_red[0]);
  }
  // the next solve's first cycle queues as many steps as this solve took
  if (conv) c->gm_guess[precond] = std::max(1, std::min(it, m));
  // the solve's own pair (b, x)
  if (conv && precond == 1 && c->pn) CK(precond_harvest_pairs(c, c->d_rhs, c->d_x, 0));
#undef CK
  if (st) {
    st->iterations = it;
    st->converged = conv ? 1 : 0;
    st->rel_residual = rel;
  }
  return conv ? AMPS_GPU_OK : AMPS_GPU_GMRES_NOT_CONVERGED;
}

// Autotuner: candidate launch shapes timed with CUDA events on the context
// stream, on scratch vectors (the operator and the sweeps have no side effects
// outside them).  ms[0..2]: operator with 64/128/256 threads per CTA;
// ms[3..5]: one 8-vector combination sweep with 76/152/304 CTAs (4 elements per thread).
amps_gpu_status field_autotune(amps_gpu_ctx* c, double* ms) {
  const long long n = 3 * c->nvc;
  cudaStream_t s = c->stream;
  cudaError_t e;
  cudaEvent_t a, b;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess)
    return set_err(c, AMPS_GPU_CUDA_ERROR, "autotune: events");
  const bool timing = c->timing;
  c->timing = false;
  amps_gpu_status st = AMPS_GPU_OK;
  auto fail = [&](cudaError_t err, const char* what) {
    st = cuda_check(c, err, what);
    return st;
  };
  double* x = c->d_x;
  double* y = c->d_w;
  if ((e = cudaMemsetAsync(x, 0, sizeof(double) * n, s)) != cudaSuccess) fail(e, "autotune");
  if ((e = cudaMemsetAsync(c->d_V, 0, sizeof(double) * n * 10, s)) != cudaSuccess) fail(e, "autotune");
  const int tbs[3] = {64, 128, 256};
  double best = 1e30;
  int best_tb = c->tune_tb;
  for (int q = 0; q < 3 && !st; q++) {
    c->tune_tb = tbs[q];
    for (int w = 0; w < 2 && !st; w++)
      if ((e = launch_matvec32(c, x, nullptr, y)) != cudaSuccess) fail(e, "autotune matvec");
    cudaEventRecord(a, s);
    for (int r = 0; r < 5 && !st; r++)
      if ((e = launch_matvec32(c, x, nullptr, y)) != cudaSuccess) fail(e, "autotune matvec");
    cudaEventRecord(b, s);
    cudaEventSynchronize(b);
    float t = 0.f;
    cudaEventElapsedTime(&t, a, b);
    if (ms) ms[q] = t / 5.0;
    if (t < best) { best = t; best_tb = tbs[q]; }
  }
  c->tune_tb = best_tb;
  const int caps[3] = {76, 152, 304};
  // the sweep: x += sum of 8 pair vectors times coefficients (k_combine_ff),
  // the shape of the solve's grid-stride vector passes
  GmState* gs = reinterpret_cast<GmState*>(c->d_red + kGmOffset);
  const int eight = 8;
  if ((e = cudaMemcpyAsync(&gs->jj, &eight, sizeof(int), cudaMemcpyHostToDevice, s)) != cudaSuccess)
    fail(e, "autotune");
  if ((e = cudaMemsetAsync(gs->y, 0, sizeof(gs->y), s)) != cudaSuccess) fail(e, "autotune");
  const float* Vf = reinterpret_cast<const float*>(c->d_V);
  best = 1e30;
  int best_cap = c->tune_red;
  for (int q = 0; q < 3 && !st; q++) {
    const unsigned gr = gridr(n, caps[q], 4);
    launch_combine_ff(s, gr, n, Vf, gs->y, &gs->jj, 8, nullptr, x);
    cudaEventRecord(a, s);
    for (int r = 0; r < 5; r++) launch_combine_ff(s, gr, n, Vf, gs->y, &gs->jj, 8, nullptr, x);
    cudaEventRecord(b, s);
    if ((e = cudaEventSynchronize(b)) != cudaSuccess) fail(e, "autotune sweep");
    float t = 0.f;
    cudaEventElapsedTime(&t, a, b);
    if (ms) ms[3 + q] = t / 5.0;
    if (t < best) { best = t; best_cap = caps[q]; }
  }
  c->tune_red = best_cap;
  c->tune_ept = 4;
  c->timing = timing;
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (!st) st = cuda_check(c, cudaGetLastError(), "autotune");
  return st;
}

cudaError_t launch_add(amps_gpu_ctx* c, const double* a, const double* b, double* o, long long n) {
  k_add<<<gridr(n), 256, 0, c->stream>>>(n, a, b, o);
  return cudaGetLastError();
}
