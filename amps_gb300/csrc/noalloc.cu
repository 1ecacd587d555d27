// ECSIM current / mass-matrix deposition that allocates no device memory.
//
// Who needs it: host codes that may not call cudaMalloc or cudaFree through a
// library -- one whose device memory is owned by its framework's pool
// allocator, or one that must not stall its other streams in the middle of a
// step (cudaFree synchronises the whole device).  They pass their own device
// buffers for the inputs and outputs; the per-block field stencils and
// per-cell partial sums that the deposition needs in between live in one
// file-scope __device__ array instead.
//
// Limits and sharing:
//   * the scratch array holds a mesh of at most kMaxBlocks = 16 blocks of 8^3
//     cells (8192 cells); larger meshes are rejected with AMPS_GPU_INVALID_ARG;
//   * the array (11.1 MiB) stays resident on every GPU that loads the library
//     until the process exits;
//   * every call uses the same array: two calls that overlap on the GPU (on
//     different streams, or from different host threads without ordering)
//     race on it.  Each call writes all scratch it reads before reading it
//     (a block whose stencil copy timed out fills its cells' partials with
//     NaN), so no state leaks from one call into the next;
//   * the first call on a device resolves the array's device address with
//     cudaGetSymbolAddress, which must not run while a stream of that device
//     is being captured.
//   * the caller's current device is restored before the call returns.
#include <cuda_runtime.h>

#include <mutex>

#include "common.cuh"
#include "deposit_core.cuh"

namespace {

constexpr int kMaxBlocks = 16;
constexpr long long kMaxCells = (long long)kMaxBlocks * AMPS_CPB;
constexpr size_t kStencilBytes = (size_t)kMaxBlocks * AMPS_SC * AMPS_DEP_STRIDE * sizeof(float);
constexpr size_t kCellMBytes = (size_t)kMaxCells * AMPS_CELLM * sizeof(float);
constexpr size_t kCellJBytes = (size_t)kMaxCells * 24 * sizeof(float);
constexpr size_t kScratchBytes = kStencilBytes + kCellMBytes + kCellJBytes;
static_assert(kStencilBytes % 256 == 0 && kCellMBytes % 256 == 0, "scratch sub-array alignment");

// The scratch.  In host code this name is only a handle: its device address
// comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_deposit_scratch[kScratchBytes];
// bounded-wait bookkeeping of the stencil staging (device code names it directly)
static __device__ unsigned long long g_na_flags[4];

constexpr int kMaxDevices = 64;
unsigned char* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_setup_mu;

// (slot, cell, weight monomial) entries of the corner assembly grouped by slot,
// and the table index of the corner inside each of its 8 cells (the same tables
// the context path builds at run time).
struct NaEntry {
  unsigned char slot, cell, mono, pad;
};
__constant__ NaEntry c_na_asm[64] = {
    {0, 0, 0, 0}, {0, 1, 2, 0}, {0, 2, 6, 0}, {0, 3, 8, 0}, {0, 4, 18, 0}, {0, 5, 20, 0},
    {0, 6, 24, 0}, {0, 7, 26, 0}, {1, 1, 1, 0}, {1, 3, 7, 0}, {1, 5, 19, 0}, {1, 7, 25, 0},
    {2, 0, 1, 0}, {2, 2, 7, 0}, {2, 4, 19, 0}, {2, 6, 25, 0}, {3, 2, 3, 0}, {3, 3, 5, 0},
    {3, 6, 21, 0}, {3, 7, 23, 0}, {4, 3, 4, 0}, {4, 7, 22, 0}, {5, 2, 4, 0}, {5, 6, 22, 0},
    {6, 0, 3, 0}, {6, 1, 5, 0}, {6, 4, 21, 0}, {6, 5, 23, 0}, {7, 1, 4, 0}, {7, 5, 22, 0},
    {8, 0, 4, 0}, {8, 4, 22, 0}, {9, 4, 9, 0}, {9, 5, 11, 0}, {9, 6, 15, 0}, {9, 7, 17, 0},
    {10, 5, 10, 0}, {10, 7, 16, 0}, {11, 4, 10, 0}, {11, 6, 16, 0}, {12, 6, 12, 0}, {12, 7, 14, 0},
    {13, 7, 13, 0}, {14, 6, 13, 0}, {15, 4, 12, 0}, {15, 5, 14, 0}, {16, 5, 13, 0}, {17, 4, 13, 0},
    {18, 0, 9, 0}, {18, 1, 11, 0}, {18, 2, 15, 0}, {18, 3, 17, 0}, {19, 1, 10, 0}, {19, 3, 16, 0},
    {20, 0, 10, 0}, {20, 2, 16, 0}, {21, 2, 12, 0}, {21, 3, 14, 0}, {22, 3, 13, 0}, {23, 2, 13, 0},
    {24, 0, 12, 0}, {24, 1, 14, 0}, {25, 1, 13, 0}, {26, 0, 13, 0}};
__constant__ unsigned char c_na_corner[8] = {0, 1, 3, 2, 4, 5, 7, 6};

struct NaMesh {
  int nbx, nby, nbz;
  __device__ __forceinline__ int nx() const { return 8 * nbx; }
  __device__ __forceinline__ int ny() const { return 8 * nby; }
  __device__ __forceinline__ int nz() const { return 8 * nbz; }
  // global periodic corner index of block-local (i,j,k), i,j,k in [-8,16)
  __device__ __forceinline__ long long global(int b, int i, int j, int k) const {
    const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
    const int I = ((bx * 8 + i) % nx() + nx()) % nx();
    const int J = ((by * 8 + j) % ny() + ny()) % ny();
    const int K = ((bz * 8 + k) % nz() + nz()) % nz();
    return (long long)I + (long long)nx() * (J + (long long)ny() * K);
  }
  // block-owned id of the same corner / cell
  __device__ __forceinline__ long long owned(int b, int i, int j, int k) const {
    const long long g = global(b, i, j, k);
    const int I = (int)(g % nx()), J = (int)((g / nx()) % ny()), K = (int)(g / ((long long)nx() * ny()));
    const int bb = (I >> 3) + nbx * ((J >> 3) + nby * (K >> 3));
    return (long long)bb * AMPS_CPB + (I & 7) + 8 * ((J & 7) + 8 * (K & 7));
  }
};

__global__ void k_na_pack(NaMesh m, const double* __restrict__ Bg, float* __restrict__ st) {
  const int b = blockIdx.x;
  for (int s = threadIdx.x; s < AMPS_SC; s += blockDim.x) {
    const int i = s % 9, j = (s / 9) % 9, k = s / 81;
    const long long g = m.global(b, i, j, k);
    reinterpret_cast<float4*>(st)[(size_t)b * AMPS_SC + s] =
        make_float4((float)Bg[3 * g], (float)Bg[3 * g + 1], (float)Bg[3 * g + 2], 0.f);
  }
}

struct NaArgs {
  const int* start;
  const float* u;
  const float* v;
  const uint8_t* sp;
  long long n;
  const float* stencil;
  float* cellM;
  float* cellJ;
  double* energy;
  float inv_vol;
  SpeciesTab st;
};

constexpr int kNaWarps = 8;

__global__ void __launch_bounds__(256) k_na_deposit(NaArgs a) {
  extern __shared__ __align__(16) float4 s_dyn[];
  float4* s_dep = s_dyn;
  float* s_rec = reinterpret_cast<float*>(s_dyn + AMPS_SC);
  __shared__ __align__(8) uint64_t bar;
  __shared__ double s_en[kNaWarps];
  const int b = blockIdx.x, k = blockIdx.y;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (!stage_stencils(&bar, s_dep, a.stencil + (size_t)b * AMPS_SC * AMPS_DEP_STRIDE,
                      AMPS_SC * AMPS_DEP_STRIDE * sizeof(float), nullptr, nullptr, 0,
                      g_na_flags)) {
    // the staging copy never completed: this CTA's cells get NaN partials
    // (so J and M are NaN where they contribute, never a previous call's
    // values) and the energy output is NaN
    const float qnan = __int_as_float(0x7fc00000);
    const long long c0 = (long long)b * AMPS_CPB + (long long)AMPS_NC * AMPS_NC * k;
    for (int t = threadIdx.x; t < AMPS_NC * AMPS_NC * AMPS_CELLM; t += blockDim.x)
      a.cellM[c0 * AMPS_CELLM + t] = qnan;
    for (int t = threadIdx.x; t < AMPS_NC * AMPS_NC * 24; t += blockDim.x) a.cellJ[c0 * 24 + t] = qnan;
    if (threadIdx.x == 0) *a.energy = __longlong_as_double(0x7ff8000000000000LL);
    return;
  }
  float* rec = s_rec + wid * kFields * kFS;
  int fA, fB;
  lane_fields(lane, fA, fB);
  FF en{0.f, 0.f};
  const int j = wid;
  for (int i = 0; i < AMPS_NC; i++) {
    const long long cid = (long long)b * AMPS_CPB + i + AMPS_NC * (j + AMPS_NC * k);
    const int b0 = a.start[cid], n0 = a.start[cid + 1] - b0;
    Tile tile;
    tile.zero();
    for (int q0 = 0; q0 < n0; q0 += 32) {
      const long long p = b0 + q0 + lane;
      const bool act = q0 + lane < n0;
      // positions past the cell's particles stage zero weight at the cell centre
      float u[3] = {i + 0.5f, j + 0.5f, k + 0.5f}, v[3] = {0.f, 0.f, 0.f};
      int s = 0;
      if (act) {
#pragma unroll
        for (int d = 0; d < 3; d++) { u[d] = a.u[d * a.n + p]; v[d] = a.v[d * a.n + p]; }
        s = a.sp[p];
      }
      stage_fields<kFS>(rec, lane, s_dep, u[0], u[1], u[2], v[0], v[1], v[2], s, act ? 1.0f : 0.f,
                        i, j, k, a.st, a.inv_vol, en);
      __syncwarp();
      tile.accumulate<kFS>(rec, (min(32, n0 - q0) + 3) & ~3, fA, fB);
      __syncwarp();
    }
    tile.flush(lane, a.cellM, a.cellJ, cid);
  }
  reduce_energy(ff_value(en), s_en, a.energy);
}

__global__ void __launch_bounds__(256) k_na_assemble(NaMesh m, long long ncor,
                                                     const float* __restrict__ cellM,
                                                     const float* __restrict__ cellJ,
                                                     double inv_vol, double* __restrict__ M,
                                                     double* __restrict__ J) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncor) return;
  const int b = (int)(c / AMPS_CPB), l = (int)(c % AMPS_CPB);
  const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
  const long long g = m.global(b, i, j, k);
  long long cell[8];
#pragma unroll
  for (int co = 0; co < 8; co++)
    cell[co] = m.owned(b, i - (co & 1), j - ((co >> 1) & 1), k - ((co >> 2) & 1));
  float acc[9];
  int cur = c_na_asm[0].slot;
#pragma unroll
  for (int e = 0; e < 9; e++) acc[e] = 0.f;
  for (int t = 0; t < 64; t++) {
    const NaEntry en = c_na_asm[t];
    if (en.slot != cur) {
#pragma unroll
      for (int e = 0; e < 9; e++) {
        M[243 * g + cur * 9 + e] = widen(acc[e]);
        acc[e] = 0.f;
      }
      cur = en.slot;
    }
    const float* src = cellM + cellM_at(cell[en.cell], en.mono * 9);
#pragma unroll
    for (int e = 0; e < 9; e++) acc[e] += src[e];
  }
#pragma unroll
  for (int e = 0; e < 9; e++) M[243 * g + cur * 9 + e] = widen(acc[e]);
  float jj[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int co = 0; co < 8; co++) {
    const float* src = cellJ + cellJ_at(cell[co], c_na_corner[co] * 3);
    jj[0] += src[0];
    jj[1] += src[1];
    jj[2] += src[2];
  }
#pragma unroll
  for (int d = 0; d < 3; d++) J[3 * g + d] = widen(jj[d]) * inv_vol;
}

// Resolves the scratch address on `dev` (current) once; 0 on success.
cudaError_t setup_device(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_deposit_scratch);
    if (e != cudaSuccess) return e;
    const int smem = (int)(AMPS_SC * sizeof(float4) + kNaWarps * kFields * kFS * sizeof(float));
    e = cudaFuncSetAttribute(k_na_deposit, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

}  // namespace

namespace {

amps_gpu_status deposit_noalloc(const amps_gpu_config* cfg, long long n, const int32_t* d_cell_start,
                                const float* d_u, const float* d_v, const uint8_t* d_spec,
                                const double* d_B_corner, double* d_J, double* d_M,
                                double* d_energy, void* stream) {
  if (!cfg || n < 0 || !d_cell_start || !d_B_corner || !d_J || !d_M || !d_energy ||
      (n > 0 && (!d_u || !d_v || !d_spec)))
    return AMPS_GPU_INVALID_ARG;
  if (cfg->nbx <= 0 || cfg->nby <= 0 || cfg->nbz <= 0 || cfg->nspec <= 0 ||
      cfg->nspec > AMPS_GPU_MAX_SPECIES || cfg->dt <= 0.0 || cfg->dx[0] <= 0 || cfg->dx[1] <= 0 ||
      cfg->dx[2] <= 0)
    return AMPS_GPU_INVALID_ARG;
  for (int s = 0; s < cfg->nspec; s++)
    if (cfg->mass[s] <= 0.0) return AMPS_GPU_INVALID_ARG;
  const long long nb = (long long)cfg->nbx * cfg->nby * cfg->nbz;
  if (nb > kMaxBlocks) return AMPS_GPU_INVALID_ARG;  // larger than the static scratch
  if (n > (1LL << 31) - 1) return AMPS_GPU_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return AMPS_GPU_NO_DEVICE;
  if (cfg->device < 0 || cfg->device >= ndev || cfg->device >= kMaxDevices)
    return AMPS_GPU_INVALID_ARG;
  if (cudaSetDevice(cfg->device) != cudaSuccess) return AMPS_GPU_CUDA_ERROR;
  unsigned char* base = nullptr;
  if (setup_device(cfg->device, &base) != cudaSuccess) return AMPS_GPU_CUDA_ERROR;
  float* stencil = reinterpret_cast<float*>(base);
  float* cellM = reinterpret_cast<float*>(base + kStencilBytes);
  float* cellJ = reinterpret_cast<float*>(base + kStencilBytes + kCellMBytes);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const NaMesh m{cfg->nbx, cfg->nby, cfg->nbz};
  const long long ncor = nb * AMPS_CPB;
  if (cudaMemsetAsync(d_energy, 0, sizeof(double), s) != cudaSuccess) return AMPS_GPU_CUDA_ERROR;
  k_na_pack<<<(unsigned)nb, 256, 0, s>>>(m, d_B_corner, stencil);
  NaArgs a;
  a.start = d_cell_start;
  a.u = d_u;
  a.v = d_v;
  a.sp = d_spec;
  a.n = n;
  a.stencil = stencil;
  a.cellM = cellM;
  a.cellJ = cellJ;
  a.energy = d_energy;
  a.inv_vol = (float)(1.0 / (cfg->dx[0] * cfg->dx[1] * cfg->dx[2]));
  for (int q = 0; q < cfg->nspec; q++) {
    a.st.qdt2m[q] = (float)(0.5 * (cfg->charge[q] * cfg->dt / cfg->mass[q]));
    a.st.qw[q] = (float)(cfg->charge[q] * cfg->weight[q]);
    const double ke = 0.5 * cfg->mass[q] * cfg->weight[q];
    a.st.keh[q] = (float)ke;
    a.st.kel[q] = (float)(ke - (double)a.st.keh[q]);
  }
  const size_t smem = AMPS_SC * sizeof(float4) + kNaWarps * kFields * kFS * sizeof(float);
  k_na_deposit<<<dim3((unsigned)nb, AMPS_NC), kNaWarps * 32, smem, s>>>(a);
  const double inv_vol = 1.0 / (cfg->dx[0] * cfg->dx[1] * cfg->dx[2]);
  k_na_assemble<<<(unsigned)((ncor + 255) / 256), 256, 0, s>>>(m, ncor, cellM, cellJ, inv_vol,
                                                               d_M, d_J);
  return cudaGetLastError() == cudaSuccess ? AMPS_GPU_OK : AMPS_GPU_CUDA_ERROR;
}

}  // namespace

extern "C" amps_gpu_status amps_gpu_update_j_mass_matrix_noalloc(
    const amps_gpu_config* cfg, long long n, const int32_t* d_cell_start, const float* d_u,
    const float* d_v, const uint8_t* d_spec, const double* d_B_corner, double* d_J, double* d_M,
    double* d_energy, void* stream) {
  // the call selects cfg->device; the host thread's current device is the
  // caller's, so it is put back on every return path
  int prev = -1;
  const bool had = cudaGetDevice(&prev) == cudaSuccess;
  const amps_gpu_status st = deposit_noalloc(cfg, n, d_cell_start, d_u, d_v, d_spec, d_B_corner,
                                             d_J, d_M, d_energy, stream);
  if (had) {
    int now = -1;
    if (cudaGetDevice(&now) == cudaSuccess && now != prev) cudaSetDevice(prev);
  }
  return st;
}
