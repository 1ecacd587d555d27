// Batched relativistic test-particle tracing in a dipole + uniform field.
//
// Step: BorisStep of srcEarth/gridless/GridlessParticleMovers.cpp:781-801
// (half drift, momentum rotation with t = q dt B/(2 gamma m), s = 2t/(1+t^2),
// half drift with the new gamma); field Dipole::GetB_Tesla
// (srcEarth/gridless/DipoleInterface.h:99-126) plus a uniform field; step size
// dt = min(dt_max, dphi_max / omega_g) (CutoffRigidityGridless.cpp:1190-1197);
// a particle stops at r < r_in, r > r_out or after max_steps.
//
// One persistent kernel: every lane owns one particle; when lanes finish, the
// warp refills them from a global queue with one atomic per warp (warp-level
// compaction), so uneven lifetimes do not idle lanes.  State is carried in
// normalised units (x / R_E, p / (m c), t c / R_E, B / B_eq) so the FP32
// variant keeps full range; the host converts SI at the boundary.  The FP32
// variant accumulates positions with compensated (Kahan) sums: a half drift is
// ~1e-2 of |x|, so plain FP32 sums would lose ~1e-5 of every displacement.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "ptx.cuh"

namespace {

constexpr double kC = 299792458.0;
constexpr int kRefill = 16;  // steps between refill checks

template <class T>
struct TraceArgs {
  T* x; T* y; T* z; T* px; T* py; T* pz;
  int32_t* status;
  int64_t* steps;
  long long n;
  unsigned long long* queue;     // next particle index
  unsigned long long* total;     // total steps
  unsigned long long* flags;     // [0] iteration cap reached
  T kq;                          // q B_eq R_E / (m c) (signed)
  T ext[3];                      // uniform field / B_eq
  T r_in2, r_out2;
  T dphi, dt_max;
  long long max_steps;
  long long iter_cap;
};

template <class T>
__device__ __forceinline__ T rsq(T v);
template <>
__device__ __forceinline__ float rsq<float>(float v) { return rsqrtf(v); }
template <>
__device__ __forceinline__ double rsq<double>(double v) { return rsqrt(v); }

template <class T>
__device__ __forceinline__ void field(const TraceArgs<T>& a, T x, T y, T z, T& bx, T& by, T& bz) {
  const T r2 = x * x + y * y + z * z;
  const T ir = rsq<T>(r2);
  const T ir2 = ir * ir;
  const T ir3 = ir2 * ir;
  const T ir5 = ir3 * ir2;
  const T mdotr = z;  // moment along +z with unit strength (B_eq R_E^3 in these units)
  bx = T(3) * x * mdotr * ir5 + a.ext[0];
  by = T(3) * y * mdotr * ir5 + a.ext[1];
  bz = T(3) * z * mdotr * ir5 - ir3 + a.ext[2];
}

// x += d with a running compensation c (FP32 only; FP64 sums are plain)
template <class T>
__device__ __forceinline__ void comp_add(T& x, T& c, T d) {
  if constexpr (sizeof(T) == 4) {
    const T yv = d - c;
    const T t = x + yv;
    c = (t - x) - yv;
    x = t;
  } else {
    x += d;
  }
}

template <class T>
__global__ void __launch_bounds__(256) k_trace(TraceArgs<T> a) {
  const int lane = threadIdx.x & 31;
  long long idx = -1;
  T x = 0, y = 0, z = 0, px = 0, py = 0, pz = 0;
  T cx = 0, cy = 0, cz = 0;  // position compensation (FP32)
  long long st = 0;
  unsigned long long my_total = 0;
  bool queue_done = false;
  for (long long iter = 0;; iter++) {
    if (iter >= a.iter_cap) {
      if (lane == 0) atomicAdd(a.flags, 1ull);
      break;
    }
    // refill finished lanes (one atomic per warp)
    const bool need = idx < 0;
    const unsigned needm = __ballot_sync(0xffffffffu, need);
    if (needm && !queue_done) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(a.queue, (unsigned long long)__popc(needm));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (base >= (unsigned long long)a.n) queue_done = true;
      if (need) {
        const unsigned long long mine = base + __popc(needm & lanemask_lt());
        if (mine < (unsigned long long)a.n) {
          idx = (long long)mine;
          x = a.x[idx]; y = a.y[idx]; z = a.z[idx];
          px = a.px[idx]; py = a.py[idx]; pz = a.pz[idx];
          cx = cy = cz = T(0);
          st = 0;
        }
      }
    }
    if (__ballot_sync(0xffffffffu, idx >= 0) == 0) break;
    int status = -1;
    if (idx >= 0) {
#pragma unroll 1
      for (int k = 0; k < kRefill; k++) {
        T bx, by, bz;
        field(a, x, y, z, bx, by, bz);
        const T bm = sqrt(bx * bx + by * by + bz * bz);
        const T g = sqrt(T(1) + px * px + py * py + pz * pz);
        T dt = a.dt_max;
        const T om = fabs(a.kq) * bm / g;
        if (om > T(0) && a.dphi / om < dt) dt = a.dphi / om;
        const T ig = T(1) / g;
        comp_add(x, cx, T(0.5) * dt * px * ig);
        comp_add(y, cy, T(0.5) * dt * py * ig);
        comp_add(z, cz, T(0.5) * dt * pz * ig);
        const T f = a.kq * dt * T(0.5) * ig;
        const T tx = f * bx, ty = f * by, tz = f * bz;
        const T sfac = T(2) / (T(1) + tx * tx + ty * ty + tz * tz);
        const T qx = px + (py * tz - pz * ty);
        const T qy = py + (pz * tx - px * tz);
        const T qz = pz + (px * ty - py * tx);
        px += sfac * (qy * tz - qz * ty);
        py += sfac * (qz * tx - qx * tz);
        pz += sfac * (qx * ty - qy * tx);
        const T ig2 = T(1) / sqrt(T(1) + px * px + py * py + pz * pz);
        comp_add(x, cx, T(0.5) * dt * px * ig2);
        comp_add(y, cy, T(0.5) * dt * py * ig2);
        comp_add(z, cz, T(0.5) * dt * pz * ig2);
        st++;
        const T r2 = x * x + y * y + z * z;
        if (r2 < a.r_in2) { status = 1; break; }
        if (r2 > a.r_out2) { status = 2; break; }
        if (st >= a.max_steps) { status = 0; break; }
      }
      if (status >= 0) {
        a.x[idx] = x; a.y[idx] = y; a.z[idx] = z;
        a.px[idx] = px; a.py[idx] = py; a.pz[idx] = pz;
        a.status[idx] = status;
        a.steps[idx] = st;
        my_total += (unsigned long long)st;
        idx = -1;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) my_total += __shfl_xor_sync(0xffffffffu, my_total, o);
  if (lane == 0 && my_total) atomicAdd(a.total, my_total);
}

template <class T>
amps_gpu_status run_trace(long long n, double* x, double* p, int32_t* status, int64_t* steps,
                          double q, double m0, double b_eq, double r_e, const double* b_ext,
                          double r_in, double r_out, long long max_steps, double dphi_max,
                          double dt_max, long long* total_steps, double* kernel_ms) {
  const double pscale = 1.0 / (m0 * kC);
  std::vector<T> h[6];
  for (auto& v : h) v.resize((size_t)n);
  for (long long i = 0; i < n; i++) {
    for (int d = 0; d < 3; d++) {
      h[d][(size_t)i] = (T)(x[3 * i + d] / r_e);
      h[3 + d][(size_t)i] = (T)(p[3 * i + d] * pscale);
    }
  }
  T* d[6] = {nullptr};
  int32_t* d_st = nullptr;
  int64_t* d_steps = nullptr;
  unsigned long long* d_ctl = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  auto cleanup = [&]() {
    for (auto& ptr : d) cudaFree(ptr);
    cudaFree(d_st); cudaFree(d_steps); cudaFree(d_ctl);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
  };
  bool ok = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess;
  for (int k = 0; k < 6 && ok; k++) ok = cudaMalloc(&d[k], sizeof(T) * std::max(n, 1LL)) == cudaSuccess;
  ok = ok && cudaMalloc(&d_st, sizeof(int32_t) * std::max(n, 1LL)) == cudaSuccess;
  ok = ok && cudaMalloc(&d_steps, sizeof(int64_t) * std::max(n, 1LL)) == cudaSuccess;
  ok = ok && cudaMalloc(&d_ctl, sizeof(unsigned long long) * 4) == cudaSuccess;
  ok = ok && cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
  for (int k = 0; k < 6 && ok; k++)
    ok = cudaMemcpyAsync(d[k], h[k].data(), sizeof(T) * n, cudaMemcpyHostToDevice, s) == cudaSuccess;
  ok = ok && cudaMemsetAsync(d_ctl, 0, sizeof(unsigned long long) * 4, s) == cudaSuccess;
  if (!ok) {
    cleanup();
    return AMPS_GPU_CUDA_ERROR;
  }
  TraceArgs<T> a;
  a.x = d[0]; a.y = d[1]; a.z = d[2]; a.px = d[3]; a.py = d[4]; a.pz = d[5];
  a.status = d_st; a.steps = d_steps; a.n = n;
  a.queue = d_ctl; a.total = d_ctl + 1; a.flags = d_ctl + 2;
  a.kq = (T)(q * b_eq * r_e / (m0 * kC));
  for (int k = 0; k < 3; k++) a.ext[k] = (T)(b_ext ? b_ext[k] / b_eq : 0.0);
  a.r_in2 = (T)((r_in / r_e) * (r_in / r_e));
  a.r_out2 = (T)((r_out / r_e) * (r_out / r_e));
  a.dphi = (T)dphi_max;
  a.dt_max = (T)(dt_max * kC / r_e);
  a.max_steps = max_steps;
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_trace<T>, 256, 0);
  if (per_sm < 1) per_sm = 1;
  const int grid = nsm * per_sm;
  const long long warps = (long long)grid * 8;
  // every warp finishes at most ceil(n/warps)+1 particles, each in at most
  // ceil(max_steps/kRefill) iterations (plus one refill iteration each)
  a.iter_cap = ((n + warps - 1) / warps + 2) * ((max_steps + kRefill - 1) / kRefill + 2) + 16;
  cudaEventRecord(e0, s);
  k_trace<T><<<grid, 256, 0, s>>>(a);
  cudaEventRecord(e1, s);
  cudaError_t err = cudaStreamSynchronize(s);
  if (err != cudaSuccess) {
    cleanup();
    return AMPS_GPU_CUDA_ERROR;
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  if (kernel_ms) *kernel_ms = ms;
  unsigned long long ctl[4];
  cudaMemcpy(ctl, d_ctl, sizeof(ctl), cudaMemcpyDeviceToHost);
  for (int k = 0; k < 6; k++)
    cudaMemcpy(h[k].data(), d[k], sizeof(T) * n, cudaMemcpyDeviceToHost);
  cudaMemcpy(status, d_st, sizeof(int32_t) * n, cudaMemcpyDeviceToHost);
  cudaMemcpy(steps, d_steps, sizeof(int64_t) * n, cudaMemcpyDeviceToHost);
  for (long long i = 0; i < n; i++)
    for (int dd = 0; dd < 3; dd++) {
      x[3 * i + dd] = (double)h[dd][(size_t)i] * r_e;
      p[3 * i + dd] = (double)h[3 + dd][(size_t)i] / pscale;
    }
  if (total_steps) *total_steps = (long long)ctl[1];
  cleanup();
  return ctl[2] ? AMPS_GPU_DEVICE_TIMEOUT : AMPS_GPU_OK;
}

}  // namespace

extern "C" amps_gpu_status amps_gpu_trace_dipole(int device, long long n, double* x, double* p,
                                                 int32_t* status, int64_t* steps, double q,
                                                 double m0, double b_eq, double r_e,
                                                 const double* b_ext, double r_in, double r_out,
                                                 long long max_steps, double dphi_max,
                                                 double dt_max, int precision,
                                                 long long* total_steps, double* kernel_ms) {
  if (n < 0 || (n > 0 && (!x || !p || !status || !steps)) || m0 <= 0.0 || b_eq == 0.0 ||
      r_e <= 0.0 || r_in < 0.0 || r_out <= r_in || max_steps <= 0 || dphi_max <= 0.0 ||
      dt_max <= 0.0 || (precision != 0 && precision != 1))
    return AMPS_GPU_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return AMPS_GPU_NO_DEVICE;
  if (device < 0 || device >= ndev) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(device);
  if (n == 0) {
    if (total_steps) *total_steps = 0;
    return AMPS_GPU_OK;
  }
  if (precision == 0)
    return run_trace<double>(n, x, p, status, steps, q, m0, b_eq, r_e, b_ext, r_in, r_out,
                             max_steps, dphi_max, dt_max, total_steps, kernel_ms);
  return run_trace<float>(n, x, p, status, steps, q, m0, b_eq, r_e, b_ext, r_in, r_out, max_steps,
                          dphi_max, dt_max, total_steps, kernel_ms);
}
