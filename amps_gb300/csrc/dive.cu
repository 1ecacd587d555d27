// div E correction: PIC::FieldSolver::Electromagnetic::ECSIM::divECorrection
// (src/pic/pic_field_solver_ecsim.cpp:4341-4364) on periodic uniform meshes,
// the reference's own restriction (:4361-4363).  The reference exits when the
// correction is switched on (:6168-6170); the steps here follow its functions:
//   ComputeNetCharge :4690-4828 -- each particle's q w spread over the 8 cell
//     centres of CellCentered::Linear's stencil (pic_interpolation_routines.cpp:
//     820-905: i0 = -1 below half a cell, else (int)(iLoc - 0.5), weight
//     iLoc - (i0 + 0.5)), summed over blocks, divided by the cell volume; the
//     previous density is kept (UpdateOldNetCharge);
//   ComputeDivE :1474-1545 -- div E of the corner E^{n+1} at the cell centres;
//   the Poisson system of PoissonGetStencil :645-735 (7-point Laplacian on
//     the cell centres, no boundary rows on a periodic mesh) and
//     PoissonUpdateRhs :6023-6036: rhs = (-4 pi (g rho_new + (1 - g) rho_old)
//     + div E) / g with g = 0.51, zero initial guess; solved by conjugate
//     gradients on -Laplacian with the right-hand side's mean removed (the
//     periodic Laplacian's null space);
//   CorrectParticleLocation :4440-4683 -- species 0 only: at the corner
//     nearest the particle, grad phi from face differences of phi interpolated
//     bilinearly (interp2D :216-232) and the species-0 charge density (summed
//     here from the particles being corrected; the reference reads its corner
//     species moments of the last deposit); displacement -0.9 grad phi /
//     (4 pi rho_e), 0 where rho_e = 0, capped at 0.1 dx; re-binning; the net
//     charge again.
// Kernels: charge sums one warp per cell into per-warp shared sums (27 cell
// centres or 8 corners), then one FP64 atomic per touched node; div E and the
// Laplacian one thread per cell; the position correction one thread per
// particle of the list buffer, then the counting-sort rebuild.
#include <cuda_runtime.h>

#include <cmath>
#include <string>

#include "common.cuh"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kGamma = 0.51;  // PoissonUpdateRhs, pic_field_solver_ecsim.cpp:6029
constexpr double kEps = 0.9;     // CorrectParticleLocation :4589
constexpr double kLimit = 0.1;   // :4599
constexpr int kPartBlocks = 304;

struct Lat {
  int nbx, nby, nbz;
};

// cell / corner id of global lattice indices, periodic
__device__ __forceinline__ long long gid(const Lat& L, int I, int J, int K) {
  const int NX = 8 * L.nbx, NY = 8 * L.nby, NZ = 8 * L.nbz;
  I = ((I % NX) + NX) % NX;
  J = ((J % NY) + NY) % NY;
  K = ((K % NZ) + NZ) % NZ;
  const long long b = I / 8 + (long long)L.nbx * (J / 8 + (long long)L.nby * (K / 8));
  return b * AMPS_CPB + (I & 7) + 8 * ((J & 7) + 8 * (K & 7));
}

__device__ __forceinline__ void block_coords(const Lat& L, int b, int bc[3]) {
  bc[0] = b % L.nbx;
  bc[1] = (b / L.nbx) % L.nby;
  bc[2] = b / (L.nbx * L.nby);
}

struct ChargeArgs {
  Lat L;
  long long ncell;
  const int* base;
  const int* cnt;
  const float* u[3];
  const uint8_t* sp;
  const float* wc;
  double qw[AMPS_GPU_MAX_SPECIES];
  double inv_vol;
  int only;  // sum only this species; -1: all
};

// CORNERS = false: the net charge on the cell centres (cell-centred linear
// stencil); true: the charge of species `only` on the corners (corner weights)
template <bool CORNERS>
__global__ void __launch_bounds__(256) k_charge(ChargeArgs a, double* __restrict__ out) {
  __shared__ double s_acc[8][27];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long long cid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  double* acc = s_acc[wid];
  if (lane < 27) acc[lane] = 0.0;
  __syncwarp();
  if (cid >= a.ncell) return;  // the whole warp
  const int l = (int)(cid % AMPS_CPB);
  const int ci[3] = {l & 7, (l >> 3) & 7, l >> 6};
  const int b0 = a.base[cid], n = a.cnt[cid];
  for (int q = lane; q < n; q += 32) {
    const long long p = (long long)b0 + q;
    const int s = a.sp[p];
    if (a.only >= 0 && s != a.only) continue;
    const double qq = a.qw[s] * (a.wc ? (double)a.wc[p] : 1.0);
    double w[3];
    int o[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double u = (double)a.u[d][p];
      if (CORNERS) {
        w[d] = u - ci[d];
        o[d] = 0;
      } else {
        const int i0 = u < 0.5 ? -1 : (int)(u - 0.5);
        w[d] = u - ((double)i0 + 0.5);
        o[d] = i0 - ci[d] + 1;  // 0 or 1: centres ci - 1 + {0, 1, 2}
      }
    }
#pragma unroll
    for (int cc = 0; cc < 2; cc++)
#pragma unroll
      for (int bb = 0; bb < 2; bb++)
#pragma unroll
        for (int aa = 0; aa < 2; aa++) {
          const double W = (aa ? w[0] : 1.0 - w[0]) * (bb ? w[1] : 1.0 - w[1]) * (cc ? w[2] : 1.0 - w[2]);
          atomicAdd(acc + (o[0] + aa) + 3 * (o[1] + bb) + 9 * (o[2] + cc), W * qq);
        }
  }
  __syncwarp();
  if (lane < 27) {
    const double v = acc[lane];
    if (v != 0.0) {
      int bc[3];
      block_coords(a.L, (int)(cid / AMPS_CPB), bc);
      const int sh = CORNERS ? 0 : -1;
      atomicAdd(out + gid(a.L, 8 * bc[0] + ci[0] + sh + lane % 3, 8 * bc[1] + ci[1] + sh + (lane / 3) % 3,
                          8 * bc[2] + ci[2] + sh + lane / 9),
                v * a.inv_vol);
    }
  }
}

// corner order of ComputeDivE: (i,j,k) (i+1,j,k) (i+1,j+1,k) (i,j+1,k), then k+1
__constant__ int c_co[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                               {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

__global__ void __launch_bounds__(256) k_div_e(Lat L, long long ncell, const double* __restrict__ E,
                                               long long ncor, double dx0, double dx1, double dx2,
                                               double* __restrict__ dive) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int l = (int)(c % AMPS_CPB);
  int bc[3];
  block_coords(L, (int)(c / AMPS_CPB), bc);
  const int I = 8 * bc[0] + (l & 7), J = 8 * bc[1] + ((l >> 3) & 7), K = 8 * bc[2] + (l >> 6);
  long long co[8];
#pragma unroll
  for (int t = 0; t < 8; t++) co[t] = gid(L, I + c_co[t][0], J + c_co[t][1], K + c_co[t][2]);
  const int pos[3][4] = {{1, 2, 5, 6}, {2, 3, 6, 7}, {4, 5, 6, 7}};
  const int neg[3][4] = {{0, 3, 4, 7}, {0, 1, 4, 5}, {0, 1, 2, 3}};
  const double dx[3] = {dx0, dx1, dx2};
  double s = 0.0;
#pragma unroll
  for (int d = 0; d < 3; d++)
#pragma unroll
    for (int t = 0; t < 4; t++) s += (E[d * ncor + co[pos[d][t]]] - E[d * ncor + co[neg[d][t]]]) / dx[d];
  dive[c] = 0.25 * s;
}

// f = -rhs of the Poisson system (its mean is removed afterwards)
__global__ void __launch_bounds__(256) k_poisson_f(long long n, const double* __restrict__ rn,
                                                   const double* __restrict__ ro,
                                                   const double* __restrict__ dive, double* __restrict__ f) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  f[c] = -((-4.0 * kPi * (kGamma * rn[c] + (1.0 - kGamma) * ro[c]) + dive[c]) / kGamma);
}

// per-block partial sums: sum of a*b (b null: sum of a; gauss: of (dive - 4 pi
// blend)^2 with a = dive, b = rho_new, g = rho_old)
__global__ void __launch_bounds__(256) k_sum_part(long long n, const double* __restrict__ a,
                                                  const double* __restrict__ b,
                                                  const double* __restrict__ g, int mode,
                                                  double* __restrict__ part) {
  __shared__ double s[8];
  double t = 0.0;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (mode == 0) t += a[i];
    else if (mode == 1) t += a[i] * b[i];
    else {
      const double r = a[i] - 4.0 * kPi * (kGamma * b[i] + (1.0 - kGamma) * g[i]);
      t += r * r;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) u += s[w];
    part[blockIdx.x] = u;
  }
}

__global__ void k_sum_final(const double* __restrict__ part, int n, double* __restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double u = 0.0;
    for (int i = 0; i < n; i++) u += part[i];
    *out = u;
  }
}

__global__ void __launch_bounds__(256) k_add_const(long long n, double* __restrict__ x, double v) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) x[c] += v;
}

// y = -Laplacian(x), 7 points
__global__ void __launch_bounds__(256) k_neg_lap(Lat L, long long n, const double* __restrict__ x,
                                                 double c0, double c1, double c2, double* __restrict__ y) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int l = (int)(c % AMPS_CPB);
  int bc[3];
  block_coords(L, (int)(c / AMPS_CPB), bc);
  const int I = 8 * bc[0] + (l & 7), J = 8 * bc[1] + ((l >> 3) & 7), K = 8 * bc[2] + (l >> 6);
  double s = 2.0 * (c0 + c1 + c2) * x[c];
  s -= c0 * (x[gid(L, I - 1, J, K)] + x[gid(L, I + 1, J, K)]);
  s -= c1 * (x[gid(L, I, J - 1, K)] + x[gid(L, I, J + 1, K)]);
  s -= c2 * (x[gid(L, I, J, K - 1)] + x[gid(L, I, J, K + 1)]);
  y[c] = s;
}

// phi += alpha p, r -= alpha Ap
__global__ void __launch_bounds__(256) k_cg_update(long long n, double alpha, const double* __restrict__ p,
                                                   const double* __restrict__ Ap, double* __restrict__ phi,
                                                   double* __restrict__ r) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  phi[c] += alpha * p[c];
  r[c] -= alpha * Ap[c];
}

// p = r + beta p
__global__ void __launch_bounds__(256) k_cg_dir(long long n, double beta, const double* __restrict__ r,
                                                double* __restrict__ p) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c < n) p[c] = r[c] + beta * p[c];
}

struct MoveArgs {
  Lat L;
  long long n;
  float* u[3];
  const uint8_t* sp;
  int* key;
  const double* phi;
  const double* cq;
  double dx[3];
  unsigned long long* moved;
};

__device__ __forceinline__ double interp2d(double vmm, double vpm, double vpp, double vmp, double a,
                                           double b) {
  return vmm * (1 - a) * (1 - b) + vpm * a * (1 - b) + vpp * a * b + vmp * (1 - a) * b;
}

// the position correction of the species-0 entries of the list buffer, their
// new cell as key
__global__ void __launch_bounds__(256) k_dive_move(MoveArgs a) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool mv = false;
  if (i < a.n && a.key[i] >= 0 && a.sp[i] == 0) {
    mv = true;
    const int key = a.key[i];
    const int l = key % AMPS_CPB;
    int bc[3];
    block_coords(a.L, key / AMPS_CPB, bc);
    const int ci[3] = {l & 7, (l >> 3) & 7, l >> 6};
    double u[3], xr[3];
    int ic[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      u[d] = (double)a.u[d][i];
      xr[d] = u[d] - ci[d];
      ic[d] = ci[d] + (xr[d] >= 0.5 ? 1 : 0);  // round(xRel), xRel in [0, 1)
      xr[d] = xr[d] >= 0.5 ? xr[d] - 0.5 : xr[d] + 0.5;
    }
    const int I = 8 * bc[0] + ic[0], J = 8 * bc[1] + ic[1], K = 8 * bc[2] + ic[2];
    // phi of the centres ic - 1 + (a, b, c)
    auto ph = [&](int aa, int bb, int cc) { return a.phi[gid(a.L, I - 1 + aa, J - 1 + bb, K - 1 + cc)]; };
    double gp[3];
    gp[0] = interp2d(ph(1, 0, 0) - ph(0, 0, 0), ph(1, 1, 0) - ph(0, 1, 0), ph(1, 1, 1) - ph(0, 1, 1),
                     ph(1, 0, 1) - ph(0, 0, 1), xr[1], xr[2]);
    gp[1] = interp2d(ph(0, 1, 0) - ph(0, 0, 0), ph(1, 1, 0) - ph(1, 0, 0), ph(1, 1, 1) - ph(1, 0, 1),
                     ph(0, 1, 1) - ph(0, 0, 1), xr[0], xr[2]);
    gp[2] = interp2d(ph(0, 0, 1) - ph(0, 0, 0), ph(1, 0, 1) - ph(1, 0, 0), ph(1, 1, 1) - ph(1, 1, 0),
                     ph(0, 1, 1) - ph(0, 1, 0), xr[0], xr[1]);
#pragma unroll
    for (int d = 0; d < 3; d++) gp[d] /= a.dx[d];
    const double rho_e = a.cq[gid(a.L, I, J, K)];
    const double t = rho_e != 0.0 ? 1.0 / (4.0 * kPi * rho_e) : 0.0;
    double disp[3];
#pragma unroll
    for (int d = 0; d < 3; d++) disp[d] = -kEps * gp[d] * t;
    if (fabs(disp[0] / a.dx[0]) > kLimit || fabs(disp[1] / a.dx[1]) > kLimit ||
        fabs(disp[2] / a.dx[2]) > kLimit) {
      const double dl = sqrt(disp[0] * disp[0] + disp[1] * disp[1] + disp[2] * disp[2]);
#pragma unroll
      for (int d = 0; d < 3; d++) disp[d] *= kLimit * a.dx[0] / dl;
    }
    // the new position on the global lattice (cell units), periodic, then its
    // block and block-local FP32 offset
    const int N[3] = {8 * a.L.nbx, 8 * a.L.nby, 8 * a.L.nbz};
    int nb[3], nl[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      double G = 8.0 * bc[d] + u[d] + disp[d] / a.dx[d];
      if (G < 0.0) G += N[d];
      else if (G >= N[d]) G -= N[d];
      nb[d] = min((int)(G * 0.125), N[d] / 8 - 1);
      float uf = (float)(G - 8.0 * nb[d]);
      if (!(uf < 8.0f)) uf = 7.99999952f;  // the largest float below 8
      if (uf < 0.0f) uf = 0.0f;
      a.u[d][i] = uf;
      nl[d] = min((int)uf, 7);
    }
    a.key[i] = (int)((nb[0] + a.L.nbx * (nb[1] + a.L.nby * nb[2])) * AMPS_CPB + nl[0] +
                     8 * (nl[1] + 8 * nl[2]));
  }
  const unsigned m = __ballot_sync(0xffffffffu, mv);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(a.moved, (unsigned long long)__popc(m));
}

unsigned grid_n(long long n) { return (unsigned)((n + 255) / 256); }

ChargeArgs charge_args(amps_gpu_ctx* c, int only) {
  ChargeArgs a{};
  a.L = {c->cfg.nbx, c->cfg.nby, c->cfg.nbz};
  a.ncell = c->ncor;
  a.base = c->d_base;
  a.cnt = c->d_cnt;
  for (int d = 0; d < 3; d++) a.u[d] = c->d_u[c->cur][d];
  a.sp = c->d_sp[c->cur];
  a.wc = c->has_wcorr ? c->d_wc[c->cur] : nullptr;
  for (int s = 0; s < AMPS_GPU_MAX_SPECIES; s++)
    a.qw[s] = s < c->cfg.nspec ? c->cfg.charge[s] * c->cfg.weight[s] : 0.0;
  a.inv_vol = 1.0 / (c->cfg.dx[0] * c->cfg.dx[1] * c->cfg.dx[2]);
  a.only = only;
  return a;
}

}  // namespace

extern "C" amps_gpu_status amps_gpu_div_e_correction(amps_gpu_ctx* c, double tol, int maxit,
                                                     int redeposit, amps_gpu_dive_stats* st) {
  if (!c || !(tol > 0.0) || maxit <= 0)
    return set_err(c, AMPS_GPU_INVALID_ARG, "div_e_correction: bad arguments");
  if (c->amr || c->open_axes)
    return set_err(c, AMPS_GPU_INVALID_ARG,
                   "div_e_correction: periodic uniform meshes only (the reference's own "
                   "restriction, pic_field_solver_ecsim.cpp:4361-4363)");
  cudaSetDevice(c->cfg.device);
  cudaStream_t s = c->stream;
  const long long nc = c->ncor;
  cudaError_t e = cudaSuccess;
  if (!c->d_dive) {
    e = cudaMalloc(reinterpret_cast<void**>(&c->d_dive), sizeof(double) * 9 * nc);
    if (e != cudaSuccess) return cuda_check(c, e, "div_e_correction: allocation");
    c->dive_have_rho = false;
  }
  double *rn = c->d_dive, *ro = rn + nc, *dive = rn + 2 * nc, *phi = rn + 3 * nc, *f = rn + 4 * nc,
         *r = rn + 5 * nc, *pv = rn + 6 * nc, *Ap = rn + 7 * nc, *cq = rn + 8 * nc;
  double* part = c->d_red;
  double* sum = c->d_red + kPartBlocks;
  const Lat L{c->cfg.nbx, c->cfg.nby, c->cfg.nbz};
  const unsigned gw = grid_n(nc * 32);
  auto reduce = [&](const double* a, const double* b, const double* g, int mode, double* out) {
    k_sum_part<<<kPartBlocks, 256, 0, s>>>(nc, a, b, g, mode, part);
    k_sum_final<<<1, 32, 0, s>>>(part, kPartBlocks, sum);
    cudaError_t ee = cudaMemcpyAsync(c->h_red, sum, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (ee == cudaSuccess) ee = cudaStreamSynchronize(s);
    *out = c->h_red[0];
    return ee;
  };
#define CK(x)                                                   \
  do {                                                          \
    e = (x);                                                    \
    if (e != cudaSuccess) return cuda_check(c, e, #x);          \
  } while (0)
  {
    TimedLaunch t(c, "dive_charge");
    if (!c->dive_have_rho) {
      CK(cudaMemsetAsync(rn, 0, sizeof(double) * nc, s));
      k_charge<false><<<gw, 256, 0, s>>>(charge_args(c, -1), rn);
    }
    // UpdateOldNetCharge, then the net charge of the current particles
    CK(cudaMemcpyAsync(ro, rn, sizeof(double) * nc, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(rn, 0, sizeof(double) * nc, s));
    k_charge<false><<<gw, 256, 0, s>>>(charge_args(c, -1), rn);
    k_div_e<<<grid_n(nc), 256, 0, s>>>(L, nc, c->d_En, c->nvc, c->cfg.dx[0], c->cfg.dx[1], c->cfg.dx[2],
                                         dive);
  }
  CK(cudaGetLastError());
  double g_before = 0.0, g_after = 0.0, fmean = 0.0, fn2 = 0.0, rr = 0.0;
  CK(reduce(dive, rn, ro, 2, &g_before));
  // Poisson: -Laplacian(phi) = f, f = -rhs with its mean removed
  k_poisson_f<<<grid_n(nc), 256, 0, s>>>(nc, rn, ro, dive, f);
  CK(reduce(f, nullptr, nullptr, 0, &fmean));
  k_add_const<<<grid_n(nc), 256, 0, s>>>(nc, f, -fmean / (double)nc);
  CK(cudaMemsetAsync(phi, 0, sizeof(double) * nc, s));
  CK(cudaMemcpyAsync(r, f, sizeof(double) * nc, cudaMemcpyDeviceToDevice, s));
  CK(cudaMemcpyAsync(pv, f, sizeof(double) * nc, cudaMemcpyDeviceToDevice, s));
  CK(reduce(f, f, nullptr, 1, &fn2));
  rr = fn2;
  const double fn = std::sqrt(fn2);
  const double c0 = 1.0 / (c->cfg.dx[0] * c->cfg.dx[0]), c1 = 1.0 / (c->cfg.dx[1] * c->cfg.dx[1]),
               c2 = 1.0 / (c->cfg.dx[2] * c->cfg.dx[2]);
  int it = 0;
  {
    TimedLaunch t(c, "dive_poisson");
    while (it < maxit && std::sqrt(rr) > tol * fn) {
      k_neg_lap<<<grid_n(nc), 256, 0, s>>>(L, nc, pv, c0, c1, c2, Ap);
      double pap = 0.0;
      CK(reduce(pv, Ap, nullptr, 1, &pap));
      const double alpha = rr / pap;
      k_cg_update<<<grid_n(nc), 256, 0, s>>>(nc, alpha, pv, Ap, phi, r);
      double rr1 = 0.0;
      CK(reduce(r, r, nullptr, 1, &rr1));
      k_cg_dir<<<grid_n(nc), 256, 0, s>>>(nc, rr1 / rr, r, pv);
      rr = rr1;
      it++;
    }
  }
  // CorrectParticleLocation: species-0 charge on the corners, the displacement,
  // re-binning, then the net charge of the corrected particles
  CK(cudaMemsetAsync(cq, 0, sizeof(double) * nc, s));
  CK(cudaMemsetAsync(c->d_flags + 7, 0, sizeof(unsigned long long), s));
  {
    TimedLaunch t(c, "dive_move", 2);
    k_charge<true><<<gw, 256, 0, s>>>(charge_args(c, 0), cq);
    CK(particles_to_list(c));
    MoveArgs m{};
    m.L = L;
    m.n = c->np;
    const int o = c->cur ^ 1;
    for (int d = 0; d < 3; d++) {
      m.u[d] = c->d_u[o][d];
      m.dx[d] = c->cfg.dx[d];
    }
    m.sp = c->d_sp[o];
    m.key = c->d_key;
    m.phi = phi;
    m.cq = cq;
    m.moved = c->d_flags + 7;
    k_dive_move<<<grid_n(c->np), 256, 0, s>>>(m);
  }
  CK(cudaGetLastError());
  CK(rebuild_from_list(c, c->np));
  CK(cudaMemsetAsync(rn, 0, sizeof(double) * nc, s));
  k_charge<false><<<gw, 256, 0, s>>>(charge_args(c, -1), rn);
  CK(reduce(dive, rn, ro, 2, &g_after));
  CK(cudaMemcpyAsync(c->h_flags + 7, c->d_flags + 7, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  c->dive_have_rho = true;
#undef CK
  if (st) {
    st->iterations = it;
    st->rel_residual = fn > 0.0 ? std::sqrt(rr) / fn : 0.0;
    st->gauss_before = std::sqrt(g_before);
    st->gauss_after = std::sqrt(g_after);
    st->moved = (long long)c->h_flags[7];
  }
  if (redeposit) {
    amps_gpu_status ss = amps_gpu_update_j_mass_matrix(c, nullptr);
    if (ss) return ss;
  }
  return AMPS_GPU_OK;
}

// the cell arrays in the host cell order (I + NX (J + NY K), as export_fields)
extern "C" amps_gpu_status amps_gpu_export_div_e(amps_gpu_ctx* c, double* rho_new, double* rho_old,
                                                 double* div_e, double* phi) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  if (!c->d_dive) return set_err(c, AMPS_GPU_INVALID_ARG, "export_div_e: no correction has run");
  cudaSetDevice(c->cfg.device);
  const long long nc = c->ncor;
  double* src[4] = {c->d_dive, c->d_dive + nc, c->d_dive + 2 * nc, c->d_dive + 3 * nc};
  double* dst[4] = {rho_new, rho_old, div_e, phi};
  for (int q = 0; q < 4; q++) {
    amps_gpu_status st = layout_download(c, src[q], dst[q], nc, 1, false);
    if (st) return st;
  }
  return AMPS_GPU_OK;
}
