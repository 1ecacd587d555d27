// Host <-> device layout conversion of fields and moments, done on the GPU.
// A page-locked host array is read or written by the permuting kernel itself
// across the host link (no staging copy in HBM); a pageable one crosses the
// bus in one bulk copy through a device staging buffer.
//
// Host layout: interleaved per point (point*ncomp + comp); points numbered
// I + NX (J + NY K) on uniform meshes (the reference's global corner order),
// unique-corner / block*512 + local on AMR meshes.  Device layout:
// component-major (comp*n + point), points owned by blocks (b*512 + local).
// FP32 device planes (the corner mass matrix, the per-cell partials) are
// widened to FP64 on the way out and rounded on the way in.
#include <cuda_runtime.h>

#include "common.cuh"
#include "deposit_core.cuh"

namespace {

struct Perm {
  int nbx, nby;
  bool identity;
};

__device__ __forceinline__ long long dev_index(const Perm& p, long long h) {
  if (p.identity) return h;
  const long long NX = 8LL * p.nbx, NY = 8LL * p.nby;
  const int I = (int)(h % NX), J = (int)((h / NX) % NY), K = (int)(h / (NX * NY));
  const int b = (I >> 3) + p.nbx * ((J >> 3) + p.nby * (K >> 3));
  return (long long)b * AMPS_CPB + (I & 7) + 8 * ((J & 7) + 8 * (K & 7));
}

// dev[comp*n + dev(h)] = host[h*ncomp + comp]   (T = double or float on device).
// One thread per host element, in host order: a warp reads 256 consecutive
// host bytes (whole lines across the host link for a page-locked array); the
// scattered device writes stay in HBM / L2.
template <class T>
__global__ void __launch_bounds__(256) k_to_device(long long n, int ncomp, Perm p,
                                                   const double* __restrict__ host,
                                                   T* __restrict__ dev) {
  const long long total = n * ncomp;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long h = t / ncomp;
    const int cc = (int)(t - h * ncomp);
    dev[(size_t)cc * n + dev_index(p, h)] = (T)host[t];
  }
}

__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ double to_f64(float v) { return widen(v); }

// host[h*ncomp + comp] = dev[comp*n + dev(h)], one thread per host element in
// host order (coalesced writes across the host link; the link, ~190 GB/s
// device to host, bounds a page-locked download)
template <class T>
__global__ void __launch_bounds__(256) k_to_host(long long n, int ncomp, Perm p,
                                                 const T* __restrict__ dev,
                                                 double* __restrict__ host) {
  const long long total = n * ncomp;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long h = t / ncomp;
    const int cc = (int)(t - h * ncomp);
    host[t] = to_f64(dev[(size_t)cc * n + dev_index(p, h)]);
  }
}

// per-cell partials -> ProcessCell's host layout: cellJ[24] as is, cellM from the
// 27 monomial sums to the 36 corner pairs (c2 <= c1) x 9, FP64
__global__ void __launch_bounds__(256) k_cell_moments_to_host(long long ncell,
                                                              const float* __restrict__ cellJ,
                                                              const float* __restrict__ cellM,
                                                              double* __restrict__ hJ,
                                                              double* __restrict__ hM) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < ncell * 324;
       t += (long long)gridDim.x * blockDim.x) {
    const long long cl = t / 324;
    const int r = (int)(t - cl * 324), pr = r / 9, e = r - pr * 9;
    if (hM) {
      int c1 = 0;
      while ((c1 + 1) * (c1 + 2) / 2 <= pr) c1++;
      const int c2 = pr - c1 * (c1 + 1) / 2;
      hM[t] = widen(cellM[cellM_at(cl, pair_monomial(c1, c2) * 9 + e)]);
    }
    if (hJ && r < 24) hJ[cl * 24 + r] = widen(cellJ[cellJ_at(cl, r)]);
  }
}

unsigned grid_of(long long n) {
  long long g = (n + 255) / 256;
  if (g > 152LL * 32) g = 152LL * 32;
  return (unsigned)(g < 1 ? 1 : g);
}

Perm perm_of(const amps_gpu_ctx* c) { return Perm{c->cfg.nbx, c->cfg.nby, c->amr}; }

}  // namespace

// device address of a page-locked host array, or null for pageable memory
double* host_mapped(double* host) {
  cudaPointerAttributes at;
  if (!host || cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? static_cast<double*>(at.devicePointer) : nullptr;
}

namespace {

template <class T>
T* mapped(T* host) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? static_cast<T*>(at.devicePointer) : nullptr;
}

// device staging of `bytes` (grows on demand, kept with the context)
double* host_stage(amps_gpu_ctx* c, size_t bytes) {
  if (c->hstage_bytes >= bytes) return c->d_hstage;
  cudaFree(c->d_hstage);
  c->d_hstage = nullptr;
  c->hstage_bytes = 0;
  if (cudaMalloc(reinterpret_cast<void**>(&c->d_hstage), bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  c->hstage_bytes = bytes;
  return c->d_hstage;
}

}  // namespace

amps_gpu_status layout_upload(amps_gpu_ctx* c, const double* host, void* dev, long long n,
                              int ncomp, bool dev_f32) {
  if (!host) return AMPS_GPU_OK;
  const size_t bytes = sizeof(double) * (size_t)n * ncomp;
  const double* st = mapped(host);
  cudaError_t e = cudaSuccess;
  if (!st) {
    double* buf = host_stage(c, bytes);
    if (!buf) return set_err(c, AMPS_GPU_CUDA_ERROR, "layout staging allocation failed");
    e = cudaMemcpyAsync(buf, host, bytes, cudaMemcpyHostToDevice, c->stream);
    st = buf;
  }
  if (e == cudaSuccess) {
    if (dev_f32)
      k_to_device<float><<<grid_of(n * ncomp), 256, 0, c->stream>>>(n, ncomp, perm_of(c), st,
                                                                   static_cast<float*>(dev));
    else
      k_to_device<double><<<grid_of(n * ncomp), 256, 0, c->stream>>>(n, ncomp, perm_of(c), st,
                                                                    static_cast<double*>(dev));
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_check(c, e, "upload");
}

amps_gpu_status layout_download(amps_gpu_ctx* c, const void* dev, double* host, long long n,
                                int ncomp, bool dev_f32) {
  if (!host) return AMPS_GPU_OK;
  const size_t bytes = sizeof(double) * (size_t)n * ncomp;
  double* direct = mapped(host);
  double* st = direct ? direct : host_stage(c, bytes);
  if (!st) return set_err(c, AMPS_GPU_CUDA_ERROR, "layout staging allocation failed");
  if (dev_f32)
    k_to_host<float><<<grid_of(n * ncomp), 256, 0, c->stream>>>(n, ncomp, perm_of(c),
                                                               static_cast<const float*>(dev), st);
  else
    k_to_host<double><<<grid_of(n * ncomp), 256, 0, c->stream>>>(n, ncomp, perm_of(c),
                                                                static_cast<const double*>(dev), st);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && !direct) e = cudaMemcpyAsync(host, st, bytes, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_check(c, e, "download");
}

amps_gpu_status layout_cell_moments(amps_gpu_ctx* c, double* hJ, double* hM) {
  const long long nc = c->ncor;
  const size_t bj = hJ ? sizeof(double) * (size_t)nc * 24 : 0;
  const size_t bm = hM ? sizeof(double) * (size_t)nc * 324 : 0;
  // page-locked destinations are written by the kernel directly
  double* mJ = hJ ? mapped(hJ) : nullptr;
  double* mM = hM ? mapped(hM) : nullptr;
  const size_t stage = (hJ && !mJ ? bj : 0) + (hM && !mM ? bm : 0);
  double* st = stage ? host_stage(c, stage) : nullptr;
  if (stage && !st) return set_err(c, AMPS_GPU_CUDA_ERROR, "layout staging allocation failed");
  double* sJ = hJ ? (mJ ? mJ : st) : nullptr;
  double* sM = hM ? (mM ? mM : st + (hJ && !mJ ? bj / sizeof(double) : 0)) : nullptr;
  k_cell_moments_to_host<<<grid_of(nc * 324), 256, 0, c->stream>>>(nc, c->d_cellJ, c->d_cellM, sJ,
                                                                    sM);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && hJ && !mJ) e = cudaMemcpyAsync(hJ, sJ, bj, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess && hM && !mM) e = cudaMemcpyAsync(hM, sM, bm, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  return cuda_check(c, e, "download cell moments");
}
