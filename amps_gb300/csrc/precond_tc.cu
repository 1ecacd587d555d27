// BF16 tensor-core inference of the learned preconditioner on sm_103a:
// tcgen05.mma with FP32 accumulators in tensor memory, one CTA per mesh block.
//
// Each 3x3x3 convolution is an implicit GEMM: D[m][n] = sum over taps t and
// input channels k of A[m + off_t][k] * B_t[k][n], m = voxel of the padded
// 12^3 region (linear index p = x + 12 y + 144 z, a zero ring around the 10^3
// region R), off_t = dx + 12 dy + 144 dz.  Activations live in shared memory
// as BF16 planes of 8 channels, 16 bytes per voxel, so the A operand of tap t
// is the same buffer read from row m0 + off_t: a K-major, non-swizzled operand
// whose 8x16-byte core matrices are 8 consecutive voxels (stride-dimension
// offset 128 B) and whose next 8 channels are the next plane (leading-dimension
// offset = plane size).  Rows 157 .. 1692 (12 tiles of 128) cover every voxel
// of R; rows outside R are computed and dropped.
//
// Per layer one thread issues 12 tiles x 27 taps x (K/16) MMAs of 128 x N x 16
// into tensor memory (N = 32, or 16 for the 3-channel output layer), commits
// them to an mbarrier, and the four warps read their 32 accumulator lanes back
// (tcgen05.ld), convert to BF16 and overwrite the activation planes in place
// (zero on the ring), or write the owned voxels' FP32 output.
// Shared memory: 4 activation planes (110,592 B) + the three layers' BF16
// weight images (110,592 B, one bulk copy); tensor memory: 512 columns.
// Every wait is bounded; a timeout is counted in flags[2].
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "common.cuh"
#include "precond.cuh"
#include "ptx.cuh"

namespace {

constexpr int kPadV = 1728;                 // 12^3 padded voxels
constexpr int kPlane = kPadV * 16;          // bytes per 8-channel BF16 plane
constexpr int kActBytes = 4 * kPlane;       // 110,592
constexpr int kMBegin = 157;                // padded voxel (1,1,1)
constexpr int kTiles = 12;                  // rows kMBegin .. kMBegin + 1535
constexpr int kW1 = 27 * 2 * 4 * 128;       // K 16 (3 used), N 32
constexpr int kW2 = 27 * 4 * 4 * 128;       // K 32, N 32
constexpr int kW3 = 27 * 4 * 2 * 128;       // K 32, N 16 (3 used)
constexpr int kWBytes = kW1 + kW2 + kW3;    // 110,592
constexpr int kSmem = kActBytes + kWBytes + 64;
constexpr int kTmemCols = 512;
constexpr uint32_t kWait = 1u << 24;

// shared-memory matrix descriptor: no swizzle, K-major
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of tcgen05
  return d;
}

// instruction descriptor, kind::f16: BF16 A and B (K-major), FP32 D, M = 128
__host__ __device__ constexpr uint32_t idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t ad, uint64_t bd, uint32_t idesc,
                                         uint32_t accum) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(ad), "l"(bd), "r"(idesc), "r"(accum)
      : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ bool interior(int p, int& i, int& j, int& k) {
  const int pz = p / 144, py = (p / 12) % 12, px = p % 12;
  i = px - 1;
  j = py - 1;
  k = pz - 1;
  return px >= 1 && px <= 10 && py >= 1 && py <= 10 && pz >= 1 && pz <= 10;
}

__global__ void __launch_bounds__(128, 1) k_precond_tc(const float* __restrict__ x,
                                                       float* __restrict__ y,
                                                       const uint16_t* __restrict__ wimg,
                                                       unsigned long long* __restrict__ flags) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* act = smem;
  uint8_t* wsm = smem + kActBytes;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kActBytes + kWBytes);  // [0] mma, [1] weights
  uint32_t* tslot = reinterpret_cast<uint32_t*>(bar + 2);
  const int s = blockIdx.x;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
  }
  // zero the activation planes (the ring and the unused input channels stay zero)
  for (int q = tid; q < kActBytes / 16; q += blockDim.x)
    reinterpret_cast<uint4*>(act)[q] = make_uint4(0u, 0u, 0u, 0u);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tslot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    mbar_arrive_expect_tx(&bar[1], kWBytes);
    bulk_copy_g2s(wsm, wimg, kWBytes, &bar[1]);
  }
  // layer-1 input: channels 0..2 of plane 0
  const float* xs = x + (size_t)s * 1000 * 3;
  for (int v = tid; v < 1000; v += blockDim.x) {
    const int i = v % 10, j = (v / 10) % 10, k = v / 100;
    const int p = (k + 1) * 144 + (j + 1) * 12 + (i + 1);
    uint4 q;
    q.x = pack_bf16(xs[3 * v], xs[3 * v + 1]);
    q.y = pack_bf16(xs[3 * v + 2], 0.f);
    q.z = 0u;
    q.w = 0u;
    *reinterpret_cast<uint4*>(act + (size_t)p * 16) = q;
  }
  fence_async_smem();
  __syncthreads();
  bool ok = mbar_wait_bounded(&bar[1], 0, kWait);
  tc_fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t act_s = smem_u32(act), w_s = smem_u32(wsm);

  for (int L = 0; L < 3 && ok; L++) {
    const int N = L < 2 ? 32 : 16;
    const int NQ = L == 0 ? 2 : 4;  // 8-channel K chunks
    const int NG = N / 8;
    const uint32_t wbase = w_s + (L == 0 ? 0 : (L == 1 ? kW1 : kW1 + kW2));
    if (tid == 0) {
      // taps outer, tiles inner: consecutive MMAs write different accumulators
      const uint32_t id = idesc_bf16(N);
      const uint64_t adesc0 = sdesc(0, kPlane, 128);
      const uint64_t bdesc0 = sdesc(0, (uint32_t)NG * 128u, 128);
      int off = -157;  // tap (-1,-1,-1)
      for (int t = 0; t < 27; t++) {
        for (int ks = 0; ks < NQ / 2; ks++) {
          const uint64_t bd = bdesc0 | (uint64_t)(((wbase + (uint32_t)((t * NQ + 2 * ks) * NG) * 128u) >> 4) & 0x3FFFu);
          uint32_t a_addr = act_s + (uint32_t)(2 * ks) * kPlane + (uint32_t)(kMBegin + off) * 16u;
          const uint32_t acc = (t | ks) != 0 ? 1u : 0u;
#pragma unroll 4
          for (int tile = 0; tile < kTiles; tile++) {
            const uint64_t ad = adesc0 | (uint64_t)((a_addr >> 4) & 0x3FFFu);
            mma_bf16(tmem + (uint32_t)(tile * N), ad, bd, id, acc);
            a_addr += 128u * 16u;
          }
        }
        // next tap: x fastest, then y, then z
        off += 1;
        if (t % 3 == 2) off += 12 - 3;
        if (t % 9 == 8) off += 144 - 36;
      }
      mma_commit(&bar[0]);
    }
    __syncwarp();
    ok = mbar_wait_bounded(&bar[0], (uint32_t)(L & 1), kWait);
    if (!ok) break;
    tc_fence_after();
    for (int tile = 0; tile < kTiles; tile++) {
      const int m = kMBegin + tile * 128 + warp * 32 + lane;
      const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(tile * N);
      int i, j, k;
      const bool in = m < kPadV && interior(m, i, j, k);
      if (L < 2) {
        float v0[16], v1[16];
        tmem_ld16(ta, v0);
        tmem_ld16(ta + 16, v1);
        if (m < kPadV) {
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const float* src = q < 2 ? v0 + 8 * q : v1 + 8 * (q - 2);
            uint4 w4 = make_uint4(0u, 0u, 0u, 0u);
            if (in) {
              w4.x = pack_bf16(src[0], src[1]);
              w4.y = pack_bf16(src[2], src[3]);
              w4.z = pack_bf16(src[4], src[5]);
              w4.w = pack_bf16(src[6], src[7]);
            }
            *reinterpret_cast<uint4*>(act + (size_t)q * kPlane + (size_t)m * 16) = w4;
          }
        }
      } else {
        float v0[16];
        tmem_ld16(ta, v0);
        if (in && i >= 1 && i <= 8 && j >= 1 && j <= 8 && k >= 1 && k <= 8) {
          float* dst = y + ((size_t)s * 1000 + (k * 10 + j) * 10 + i) * 3;
          dst[0] = v0[0];
          dst[1] = v0[1];
          dst[2] = v0[2];
        }
      }
    }
    tc_fence_before();
    fence_async_smem();
    __syncthreads();
    tc_fence_after();
  }
  if (!ok) {
    if (tid == 0) atomicAdd(flags + 2, 1ull);
    // let outstanding MMAs and the weight copy finish before releasing memory
    mbar_wait_bounded(&bar[0], 0, kWait);
    mbar_wait_bounded(&bar[1], 0, kWait);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols)
                 : "memory");
  }
}

// BF16 operand images of the FP32 weights: layer L, tap t, K chunk q, N group g:
// core matrix of 8 rows (n = 8g + r) x 8 K elements (k = 8q + e), 128 bytes.
__global__ void k_pack_wtc(const float* __restrict__ w1, const float* __restrict__ w2,
                           const float* __restrict__ w3, uint16_t* __restrict__ img) {
  const int total = kWBytes / 2;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < total; q += gridDim.x * blockDim.x) {
    int byte = q * 2, L, cin, cout, NQ, NG;
    const float* W;
    if (byte < kW1) {
      L = 0; W = w1; cin = 3; cout = 32; NQ = 2; NG = 4;
    } else if (byte < kW1 + kW2) {
      L = 1; W = w2; cin = 32; cout = 32; NQ = 4; NG = 4; byte -= kW1;
    } else {
      L = 2; W = w3; cin = 32; cout = 3; NQ = 4; NG = 2; byte -= kW1 + kW2;
    }
    (void)L;
    const int core = byte / 128, within = byte % 128;
    const int r = within / 16, e = (within % 16) / 2;
    const int g = core % NG, tq = core / NG, qq = tq % NQ, t = tq / NQ;
    const int n = 8 * g + r, k = 8 * qq + e;
    const float v = (k < cin && n < cout) ? W[((size_t)t * cin + k) * cout + n] : 0.f;
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    img[q] = *reinterpret_cast<const uint16_t*>(&h);
  }
}

}  // namespace

cudaError_t precond_prepare_tc(PrecondState* P, cudaStream_t st) {
  P->tc_ready = false;
  if (!P->wtc) {
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&P->wtc), kWBytes);
    if (e != cudaSuccess) return e;
  }
  k_pack_wtc<<<108, 256, 0, st>>>(P->w[0], P->w[1], P->w[2], P->wtc);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) P->tc_ready = true;
  return e;
}

cudaError_t precond_forward_tc(PrecondState* P, cudaStream_t st, int S, const float* x, float* y) {
  if (!P->tc_ready || !P->flags) return cudaErrorInvalidValue;
  static unsigned long long attr_set = 0;  // per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (!((attr_set >> dev) & 1ull)) {
    cudaError_t e = cudaFuncSetAttribute(k_precond_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    if (e != cudaSuccess) return e;
    attr_set |= 1ull << dev;
  }
  k_precond_tc<<<S, 128, kSmem, st>>>(x, y, P->wtc, P->flags);
  return cudaGetLastError();
}
