// Particle restart format and checksum of the reference
// (PIC::Restart::SaveParticleData / ReadParticleData, src/pic/pic_restart.cpp:
// 248-575; GetParticleDataCheckSum :578-642):
//
//   header   the end-of-user-data marker (43 bytes, "PARTICLE-RESTART-FILE--END-
//            USER-ADDITIONAL" with its terminating zero), ParticleDataLength
//            (long int), the species' global particle weights (double each)
//   blocks   in the caller's tree order, those holding particles: the node id
//            (cAMRnodeID bytes from the caller), the particle count (int), the
//            per-cell counts ParticleNumberTable[i][j][k] (512 int, i slowest),
//            and for i, j, k the cell's particle records in reverse list order
//            (ReadParticleData pushes each at the head of the cell's list, so
//            the list comes back in its original order)
//   record   ParticleDataLength bytes laid out as the caller's build defines
//            (picParticleBasicOffset.cpp: next and prev links, velocity,
//            position, species byte, weight correction ...); the links are
//            written as zero, fields the device does not hold are zero
//
// The list order of a cell is its slot order on the device.  The checksum is
// the reference's CRC32 class (src/general/specfunc.h:438-505: polynomial
// 0x04C11DB7 MSB first, initial value 0, no final xor, in a 64-bit
// accumulator whose upper half keeps the bytes shifted out) over every
// record with zeroed links (GetParticleSignature, pic_pbuffer.cpp:1109-1123)
// in list order.  The device computes each record's CRC from zero in
// parallel and combines them with the linear "append n records" operator
// (a 32 x 32 GF(2) matrix power); the last record is replayed on the host in
// the 64-bit accumulator, which fixes the upper half (it only depends on the
// last four bytes' states).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.cuh"

namespace {

constexpr int kMarkerLen = 43;
constexpr char kMarker[kMarkerLen] = "PARTICLE-RESTART-FILE--END-USER-ADDITIONAL";
constexpr int kMaxRecord = 256;
constexpr int kChunk = 256;  // records combined per thread in the first pass

struct Layout {
  int len, off_v, off_x, off_sp, off_w;
};

// the reference's table (its 64-bit entries; the index only sees bits 24..31
// of the accumulator, so the low halves are the standard MSB-first table)
void crc_table64(unsigned long long t[256]) {
  for (int i = 0; i < 256; i++) {
    unsigned long long a = (unsigned long long)i << 24;
    for (int j = 0; j < 8; j++) a = (a & 0x80000000ull) ? (a << 1) ^ 0x04c11db7ull : a << 1;
    t[i] = a;
  }
}

// 32 x 32 GF(2) matrices as 32 column words: y = M x = XOR of col[b] for set bits b of x
struct Mat {
  uint32_t col[32];
};
uint32_t mat_apply(const Mat& m, uint32_t x) {
  uint32_t y = 0;
  for (int b = 0; b < 32; b++)
    if ((x >> b) & 1u) y ^= m.col[b];
  return y;
}
Mat mat_mul(const Mat& a, const Mat& b) {  // a * b
  Mat r;
  for (int k = 0; k < 32; k++) r.col[k] = mat_apply(a, b.col[k]);
  return r;
}
Mat mat_identity() {
  Mat r;
  for (int k = 0; k < 32; k++) r.col[k] = 1u << k;
  return r;
}
// one zero byte appended to the stream (the low 32 bits of the accumulator)
Mat zero_byte(const uint32_t lo[256]) {
  Mat r;
  for (int k = 0; k < 32; k++) {
    const uint32_t x = 1u << k;
    r.col[k] = (x << 8) ^ lo[x >> 24];
  }
  return r;
}
Mat mat_pow(Mat m, unsigned long long e) {
  Mat r = mat_identity();
  while (e) {
    if (e & 1ull) r = mat_mul(m, r);
    m = mat_mul(m, m);
    e >>= 1;
  }
  return r;
}

__device__ __forceinline__ void put_bytes(uint8_t* dst, const void* src, int n) {
  const uint8_t* s = static_cast<const uint8_t*>(src);
  for (int q = 0; q < n; q++) dst[q] = s[q];
}

// the record of particle (slot p) into rec[len] (zero elsewhere)
__device__ __forceinline__ void make_record(uint8_t* rec, const Layout& L, double x[3], const float v[3],
                                            uint8_t sp, double w) {
  for (int q = 0; q < L.len; q++) rec[q] = 0;
  const double vd[3] = {(double)v[0], (double)v[1], (double)v[2]};
  put_bytes(rec + L.off_v, vd, 24);
  put_bytes(rec + L.off_x, x, 24);
  rec[L.off_sp] = sp;
  if (L.off_w >= 0) put_bytes(rec + L.off_w, &w, 8);
}

struct PackArgs {
  const int* base;
  const int* cnt;
  const float* u[3];
  const float* v[3];
  const uint8_t* sp;
  const float* wc;           // may be null (weight 1)
  const double* origin;      // [nb*3] block origins
  const double* bdx;         // [nb*3] block cell sizes
  const long long* cell_byte;  // restart: byte of the cell's first record (reverse order)
  const long long* cell_rec;   // checksum: index of the cell's first record (list order)
  long long ncell;
  Layout L;
  uint8_t* out;              // restart bytes (may be null)
  uint32_t* crc;             // per-record CRC in list order (may be null)
};

// One warp per cell, 32 particles at a time: each lane builds its record in
// the warp's shared staging area, placed so that the staged bytes are the
// file's bytes for these records (reverse list order); the warp then stores
// them as aligned 32-bit words (bytes at the ragged ends), so one store
// instruction writes 128 contiguous bytes.  Each lane forms its record's CRC
// from the staged bytes.
constexpr int kPackThreads = 128;

__global__ void __launch_bounds__(kPackThreads) k_pack(PackArgs a) {
  extern __shared__ uint8_t s_dyn[];
  __shared__ uint32_t s_tab[256];
  if (a.crc) {
    for (int q = threadIdx.x; q < 256; q += blockDim.x) {
      uint32_t t = (uint32_t)q << 24;
      for (int j = 0; j < 8; j++) t = (t & 0x80000000u) ? (t << 1) ^ 0x04c11db7u : t << 1;
      s_tab[q] = t;
    }
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int len = a.L.len;
  uint8_t* wrec = s_dyn + (threadIdx.x >> 5) * 32 * len;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long cid = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); cid < a.ncell;
       cid += nw) {
    const int b = (int)(cid / AMPS_CPB);
    const int b0 = a.base[cid], n = a.cnt[cid];
    for (int r0 = 0; r0 < n; r0 += 32) {
      const int m = min(32, n - r0);
      if (lane < m) {
        const long long p = b0 + r0 + lane;
        double x[3];
        float v[3];
        for (int d = 0; d < 3; d++) {
          x[d] = a.origin[3 * b + d] + (double)a.u[d][p] * a.bdx[3 * b + d];
          v[d] = a.v[d][p];
        }
        uint8_t* rec = wrec + (m - 1 - lane) * len;
        make_record(rec, a.L, x, v, a.sp[p], a.wc ? (double)a.wc[p] : 1.0);
        if (a.crc) {
          uint32_t c = 0;
          for (int q = 0; q < len; q++) c = (c << 8) ^ s_tab[((c >> 24) ^ rec[q]) & 0xffu];
          a.crc[a.cell_rec[cid] + r0 + lane] = c;
        }
      }
      __syncwarp();
      if (a.out) {
        // file records n-r0-m .. n-r0-1 hold list positions r0+m-1 .. r0
        uint8_t* dst = a.out + a.cell_byte[cid] + (long long)(n - r0 - m) * len;
        const int nbytes = m * len;
        const int head = min(nbytes, (int)((4 - ((uintptr_t)dst & 3u)) & 3u));
        const int nword = (nbytes - head) >> 2;
        const int tail0 = head + 4 * nword;
        if (lane < head) dst[lane] = wrec[lane];
        if (lane < nbytes - tail0) dst[tail0 + lane] = wrec[tail0 + lane];
        uint32_t* dw = reinterpret_cast<uint32_t*>(dst + head);
        for (int w = lane; w < nword; w += 32) {
          const uint8_t* q = wrec + head + 4 * w;
          dw[w] = (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16) | ((uint32_t)q[3] << 24);
        }
      }
      __syncwarp();
    }
  }
}

// first combining pass: chunk k of kChunk records -> its CRC (records appended
// with the one-record operator M given as 32 columns)
__global__ void __launch_bounds__(256) k_crc_chunks(const uint32_t* __restrict__ crc, long long n,
                                                    const uint32_t* __restrict__ mcol,
                                                    uint32_t* __restrict__ chunk) {
  __shared__ uint32_t s_m[32];
  if (threadIdx.x < 32) s_m[threadIdx.x] = mcol[threadIdx.x];
  __syncthreads();
  const long long nch = (n + kChunk - 1) / kChunk;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nch;
       k += (long long)gridDim.x * blockDim.x) {
    uint32_t acc = 0;
    const long long e = std::min<long long>(n, (k + 1) * kChunk);
    for (long long q = k * kChunk; q < e; q++) {
      uint32_t y = 0;
      for (int b = 0; b < 32; b++)
        if ((acc >> b) & 1u) y ^= s_m[b];
      acc = y ^ crc[q];
    }
    chunk[k] = acc;
  }
}

struct UnpackArgs {
  const uint8_t* in;           // the file on the device
  const int* cnt;              // per-cell counts of the file
  const long long* cell_byte;  // byte of the cell's first record (reverse order)
  const long long* cell_rec;   // list index of the cell's first record
  const double* origin;
  const double* bdx;
  long long ncell;
  Layout L;
  int nspec;
  float* u[3];
  float* v[3];
  uint8_t* sp;
  float* wc;                   // null: no weight correction in the records
  uint32_t* id;                // null: ids not tracked
  int* key;
  int* rank;
  unsigned long long* bad;     // [0] positions outside the cell, [1] species out of range
};

__device__ __forceinline__ double get_f64(const uint8_t* p) {
  unsigned long long b = 0;
  for (int q = 7; q >= 0; q--) b = (b << 8) | p[q];
  return __longlong_as_double((long long)b);
}

// One warp per cell, 32 records at a time: the warp loads the records' bytes
// (contiguous in the file, reverse list order) into its shared staging area
// as aligned 32-bit words, then each lane parses one record into the list
// buffer in list order, with key = cell and rank = list position.
constexpr int kUnpackThreads = 128;

__global__ void __launch_bounds__(kUnpackThreads) k_unpack(UnpackArgs a) {
  extern __shared__ uint8_t s_dyn[];
  const int lane = threadIdx.x & 31;
  const int len = a.L.len;
  uint8_t* wrec = s_dyn + (threadIdx.x >> 5) * 32 * len;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long cid = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); cid < a.ncell;
       cid += nw) {
    const int n = a.cnt[cid];
    if (n == 0) continue;
    const int b = (int)(cid / AMPS_CPB), l = (int)(cid % AMPS_CPB);
    const int ci[3] = {l % AMPS_NC, (l / AMPS_NC) % AMPS_NC, l / (AMPS_NC * AMPS_NC)};
    for (int r0 = 0; r0 < n; r0 += 32) {
      const int m = min(32, n - r0);
      const uint8_t* src = a.in + a.cell_byte[cid] + (long long)(n - r0 - m) * len;
      const int nbytes = m * len;
      const int head = min(nbytes, (int)((4 - ((uintptr_t)src & 3u)) & 3u));
      const int nword = (nbytes - head) >> 2;
      const int tail0 = head + 4 * nword;
      if (lane < head) wrec[lane] = src[lane];
      if (lane < nbytes - tail0) wrec[tail0 + lane] = src[tail0 + lane];
      const uint32_t* sw = reinterpret_cast<const uint32_t*>(src + head);
      for (int w = lane; w < nword; w += 32) {
        const uint32_t v = sw[w];
        uint8_t* q = wrec + head + 4 * w;
        q[0] = (uint8_t)v;
        q[1] = (uint8_t)(v >> 8);
        q[2] = (uint8_t)(v >> 16);
        q[3] = (uint8_t)(v >> 24);
      }
      __syncwarp();
      if (lane < m) {
        const int r = r0 + lane;
        const uint8_t* rec = wrec + (m - 1 - lane) * len;
        const long long q = a.cell_rec[cid] + r;
        bool outside = false;
        for (int d = 0; d < 3; d++) {
          const double ud = (get_f64(rec + a.L.off_x + 8 * d) - a.origin[3 * b + d]) / a.bdx[3 * b + d];
          float uf = (float)ud;
          const float lo = (float)ci[d], hi = (float)(ci[d] + 1);
          if (!(ud >= lo && ud < hi)) outside = true;
          // keep the slot invariant (the offset lies in the cell's range)
          if (!(uf >= lo)) uf = lo;
          if (uf >= hi) uf = __int_as_float(__float_as_int(hi) - 1);
          a.u[d][q] = uf;
          a.v[d][q] = (float)get_f64(rec + a.L.off_v + 8 * d);
        }
        uint8_t sp = rec[a.L.off_sp];
        if (sp >= a.nspec) {
          atomicAdd(&a.bad[1], 1ull);
          sp = 0;
        }
        if (outside) atomicAdd(&a.bad[0], 1ull);
        a.sp[q] = sp;
        if (a.wc) a.wc[q] = (float)get_f64(rec + a.L.off_w);
        if (a.id) a.id[q] = (uint32_t)q;
        a.key[q] = (int)cid;
        a.rank[q] = r;
      }
      __syncwarp();
    }
  }
}

Layout layout_of(const amps_gpu_record_layout* l) {
  return Layout{l->record_length, l->off_velocity, l->off_position, l->off_species, l->off_weight};
}

bool layout_ok(const Layout& L) {
  auto in = [&](int off, int n) { return off >= 16 && off + n <= L.len; };
  if (L.len < 16 + 49 || L.len > kMaxRecord) return false;
  if (!in(L.off_v, 24) || !in(L.off_x, 24) || !in(L.off_sp, 1)) return false;
  if (L.off_w >= 0 && !in(L.off_w, 8)) return false;
  // no overlaps
  int seg[4][2] = {{L.off_v, 24}, {L.off_x, 24}, {L.off_sp, 1}, {L.off_w, L.off_w >= 0 ? 8 : 0}};
  for (int i = 0; i < 4; i++)
    for (int j = i + 1; j < 4; j++)
      if (seg[i][1] && seg[j][1] && seg[i][0] < seg[j][0] + seg[j][1] && seg[j][0] < seg[i][0] + seg[i][1])
        return false;
  return true;
}

// Host-side plan: per-cell record indices (list order) and restart byte
// positions, block headers, total size.
struct Plan {
  std::vector<int> cnt;
  std::vector<long long> cell_byte, cell_rec;
  std::vector<int> order;               // blocks in file order
  std::vector<long long> block_byte;    // header position of each written block (-1: none)
  long long header_bytes = 0, total_bytes = 0, nrec = 0;
};

amps_gpu_status make_plan(amps_gpu_ctx* c, const Layout& L, const int32_t* block_order, int id_len,
                          Plan& P) {
  const long long ncell = c->ncor;
  P.cnt.resize((size_t)ncell);
  cudaError_t e = cudaMemcpyAsync(P.cnt.data(), c->d_cnt, sizeof(int) * ncell, cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return cuda_check(c, e, "restart: counts");
  P.order.resize((size_t)c->nb);
  std::vector<char> seen((size_t)c->nb, 0);
  for (int q = 0; q < c->nb; q++) {
    const int b = block_order ? block_order[q] : q;
    if (b < 0 || b >= c->nb || seen[(size_t)b])
      return set_err(c, AMPS_GPU_INVALID_ARG, "restart: block_order is not a permutation of the blocks");
    seen[(size_t)b] = 1;
    P.order[(size_t)q] = b;
  }
  P.header_bytes = kMarkerLen + 8 + 8LL * c->cfg.nspec;
  P.cell_byte.assign((size_t)ncell, 0);
  P.cell_rec.assign((size_t)ncell, 0);
  P.block_byte.assign((size_t)c->nb, -1);
  long long pos = P.header_bytes, rec = 0;
  // checksum order: blocks in order, cells i, j, k (i slowest), list order
  for (int q = 0; q < c->nb; q++) {
    const int b = P.order[(size_t)q];
    long long tot = 0;
    for (int l = 0; l < AMPS_CPB; l++) tot += P.cnt[(size_t)b * AMPS_CPB + l];
    if (tot == 0) continue;
    P.block_byte[(size_t)b] = pos;
    pos += id_len + 4 + 4 * AMPS_CPB;
    for (int i = 0; i < 8; i++)
      for (int j = 0; j < 8; j++)
        for (int k = 0; k < 8; k++) {
          const long long cid = (long long)b * AMPS_CPB + i + 8 * (j + 8 * k);
          P.cell_rec[(size_t)cid] = rec;
          P.cell_byte[(size_t)cid] = pos;
          const int n = P.cnt[(size_t)cid];
          rec += n;
          pos += (long long)n * L.len;
        }
  }
  P.nrec = rec;
  P.total_bytes = pos;
  return AMPS_GPU_OK;
}

// block origins and cell sizes of the context's blocks
void block_geometry(amps_gpu_ctx* c, std::vector<double>& origin, std::vector<double>& bdx) {
  origin.assign((size_t)c->nb * 3, 0.0);
  bdx.assign((size_t)c->nb * 3, 0.0);
  if (c->amr) {
    std::vector<int> borg((size_t)c->nb * 3), bscale((size_t)c->nb);
    cudaMemcpy(borg.data(), c->d_borg, sizeof(int) * borg.size(), cudaMemcpyDeviceToHost);
    cudaMemcpy(bscale.data(), c->d_bscale, sizeof(int) * bscale.size(), cudaMemcpyDeviceToHost);
    for (int b = 0; b < c->nb; b++) {
      for (int d = 0; d < 3; d++) {
        origin[(size_t)(3 * b + d)] = c->cfg.x0[d] + borg[(size_t)(3 * b + d)] * c->dxf;
        bdx[(size_t)(3 * b + d)] = bscale[(size_t)b] * c->dxf;
      }
    }
  } else {
    for (int b = 0; b < c->nb; b++) {
      const int bc[3] = {b % c->cfg.nbx, (b / c->cfg.nbx) % c->cfg.nby, b / (c->cfg.nbx * c->cfg.nby)};
      for (int d = 0; d < 3; d++) {
        origin[(size_t)(3 * b + d)] = c->cfg.x0[d] + bc[d] * (AMPS_NC * c->cfg.dx[d]);
        bdx[(size_t)(3 * b + d)] = c->cfg.dx[d];
      }
    }
  }
}

// device address of page-locked host memory, or null for pageable memory
void* mapped_ptr(const void* host) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, host) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

template <class T>
T* dev_upload(const std::vector<T>& h, cudaError_t& e) {
  T* d = nullptr;
  if (e != cudaSuccess) return nullptr;
  e = cudaMalloc(reinterpret_cast<void**>(&d), sizeof(T) * std::max<size_t>(h.size(), 1));
  if (e == cudaSuccess && !h.empty()) e = cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
  return d;
}

// Pack on the device: restart bytes into out_dev and/or per-record CRCs.
amps_gpu_status run_pack(amps_gpu_ctx* c, const Layout& L, const Plan& P, uint8_t* out_dev,
                         uint32_t* crc_dev) {
  std::vector<double> origin, bdx;
  block_geometry(c, origin, bdx);
  cudaError_t e = cudaSuccess;
  double* d_origin = dev_upload(origin, e);
  double* d_bdx = dev_upload(bdx, e);
  long long* d_byte = dev_upload(P.cell_byte, e);
  long long* d_rec = dev_upload(P.cell_rec, e);
  if (e == cudaSuccess) {
    PackArgs a{};
    a.base = c->d_base;
    a.cnt = c->d_cnt;
    for (int d = 0; d < 3; d++) {
      a.u[d] = c->d_u[c->cur][d];
      a.v[d] = c->d_v[c->cur][d];
    }
    a.sp = c->d_sp[c->cur];
    a.wc = c->has_wcorr ? c->d_wc[c->cur] : nullptr;
    a.origin = d_origin;
    a.bdx = d_bdx;
    a.cell_byte = d_byte;
    a.cell_rec = d_rec;
    a.ncell = c->ncor;
    a.L = L;
    a.out = out_dev;
    a.crc = crc_dev;
    const int wpb = kPackThreads / 32;
    const long long blocks = std::max<long long>(1, std::min<long long>((c->ncor + wpb - 1) / wpb, 152LL * 32));
    k_pack<<<(unsigned)blocks, kPackThreads, (size_t)wpb * 32 * L.len, c->stream>>>(a);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  }
  cudaFree(d_origin);
  cudaFree(d_bdx);
  cudaFree(d_byte);
  cudaFree(d_rec);
  return cuda_check(c, e, "restart: pack");
}

}  // namespace

extern "C" {

amps_gpu_status amps_gpu_restart_particle_bytes(amps_gpu_ctx* c, const amps_gpu_record_layout* layout,
                                                int id_length, long long* bytes) {
  if (!c || !layout || !bytes || id_length < 0) return AMPS_GPU_INVALID_ARG;
  const Layout L = layout_of(layout);
  if (!layout_ok(L)) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: bad record layout");
  cudaSetDevice(c->cfg.device);
  Plan P;
  amps_gpu_status s = make_plan(c, L, nullptr, id_length, P);
  if (s) return s;
  *bytes = P.total_bytes;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_write_restart_particles(amps_gpu_ctx* c, const amps_gpu_record_layout* layout,
                                                 const int32_t* block_order, const void* node_ids,
                                                 int id_length, void* out, long long capacity,
                                                 long long* written) {
  if (!c || !layout || !out || id_length < 0 || (id_length > 0 && !node_ids)) return AMPS_GPU_INVALID_ARG;
  const Layout L = layout_of(layout);
  if (!layout_ok(L)) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: bad record layout");
  cudaSetDevice(c->cfg.device);
  Plan P;
  amps_gpu_status s = make_plan(c, L, block_order, id_length, P);
  if (s) return s;
  if (capacity < P.total_bytes) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: output buffer too small");
  // records are packed straight into page-locked output, else into device
  // staging copied out in one transfer; every record byte is written by the
  // device, the headers by the host afterwards
  uint8_t* direct = static_cast<uint8_t*>(mapped_ptr(out));
  uint8_t* d_out = direct;
  cudaError_t e = cudaSuccess;
  if (!direct) {
    e = cudaMalloc(reinterpret_cast<void**>(&d_out), (size_t)std::max<long long>(P.total_bytes, 1));
    if (e != cudaSuccess) return cuda_check(c, e, "restart: staging");
  }
  s = run_pack(c, L, P, d_out, nullptr);
  if (!s && !direct) {
    e = cudaMemcpy(out, d_out, (size_t)P.total_bytes, cudaMemcpyDeviceToHost);
    s = cuda_check(c, e, "restart: copy out");
  }
  if (!direct) cudaFree(d_out);
  if (s) return s;
  // header and block headers
  uint8_t* o = static_cast<uint8_t*>(out);
  std::memcpy(o, kMarker, kMarkerLen);
  const long long len = L.len;  // long int on LP64
  std::memcpy(o + kMarkerLen, &len, 8);
  for (int q = 0; q < c->cfg.nspec; q++) std::memcpy(o + kMarkerLen + 8 + 8 * q, &c->cfg.weight[q], 8);
  for (int q = 0; q < c->nb; q++) {
    const int b = P.order[(size_t)q];
    const long long hb = P.block_byte[(size_t)b];
    if (hb < 0) continue;
    uint8_t* h = o + hb;
    if (id_length) std::memcpy(h, static_cast<const uint8_t*>(node_ids) + (size_t)b * id_length, (size_t)id_length);
    int tot = 0;
    int table[AMPS_CPB];
    for (int i = 0; i < 8; i++)
      for (int j = 0; j < 8; j++)
        for (int k = 0; k < 8; k++) {
          const int n = P.cnt[(size_t)b * AMPS_CPB + i + 8 * (j + 8 * k)];
          table[i * 64 + j * 8 + k] = n;
          tot += n;
        }
    std::memcpy(h + id_length, &tot, 4);
    std::memcpy(h + id_length + 4, table, sizeof(table));
  }
  if (written) *written = P.total_bytes;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_particle_checksum(amps_gpu_ctx* c, const amps_gpu_record_layout* layout,
                                           const int32_t* block_order, unsigned long long* checksum) {
  if (!c || !layout || !checksum) return AMPS_GPU_INVALID_ARG;
  const Layout L = layout_of(layout);
  if (!layout_ok(L)) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: bad record layout");
  cudaSetDevice(c->cfg.device);
  Plan P;
  amps_gpu_status s = make_plan(c, L, block_order, 0, P);
  if (s) return s;
  *checksum = 0;
  if (P.nrec == 0) return AMPS_GPU_OK;
  unsigned long long t64[256];
  crc_table64(t64);
  uint32_t lo[256];
  for (int i = 0; i < 256; i++) lo[i] = (uint32_t)t64[i];
  const Mat M = mat_pow(zero_byte(lo), (unsigned long long)L.len);  // one record appended
  uint32_t *d_crc = nullptr, *d_chunk = nullptr, *d_m = nullptr;
  const long long nch = (P.nrec + kChunk - 1) / kChunk;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&d_crc), sizeof(uint32_t) * P.nrec);
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_chunk), sizeof(uint32_t) * nch);
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_m), sizeof(M.col));
  if (e == cudaSuccess) e = cudaMemcpy(d_m, M.col, sizeof(M.col), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    s = run_pack(c, L, P, nullptr, d_crc);
  } else {
    s = cuda_check(c, e, "restart: checksum buffers");
  }
  std::vector<uint32_t> chunk((size_t)nch);
  uint8_t last[kMaxRecord];
  if (!s) {
    // chunks over every record but the last (replayed on the host)
    const long long n1 = P.nrec - 1;
    const long long nch1 = (n1 + kChunk - 1) / kChunk;
    if (n1 > 0) {
      k_crc_chunks<<<(unsigned)std::min<long long>((nch1 + 255) / 256, 1216), 256, 0, c->stream>>>(d_crc, n1, d_m,
                                                                                                   d_chunk);
      e = cudaGetLastError();
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(chunk.data(), d_chunk, sizeof(uint32_t) * nch1, cudaMemcpyDeviceToHost, c->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    }
    s = cuda_check(c, e, "restart: checksum chunks");
    if (!s) {
      const Mat MC = mat_pow(M, kChunk);
      uint32_t acc = 0;
      for (long long k = 0; k < nch1; k++) {
        const long long nk = std::min<long long>(kChunk, n1 - k * kChunk);
        acc = mat_apply(nk == kChunk ? MC : mat_pow(M, (unsigned long long)nk), acc) ^ chunk[(size_t)k];
      }
      // the last record in checksum order: the last slot of the last non-empty
      // cell of the last block (in file order) holding particles
      long long last_cell = -1;
      for (long long cid = 0; cid < c->ncor; cid++) {
        const int n = P.cnt[(size_t)cid];
        if (n > 0 && P.cell_rec[(size_t)cid] + n == P.nrec) last_cell = cid;
      }
      const int last_rank = P.cnt[(size_t)last_cell] - 1;
      std::vector<double> origin, bdx;
      block_geometry(c, origin, bdx);
      int b0 = 0;
      float uu[3], vv[3], wcv = 1.0f;
      uint8_t spv = 0;
      e = cudaMemcpy(&b0, c->d_base + last_cell, sizeof(int), cudaMemcpyDeviceToHost);
      const long long slot = (long long)b0 + last_rank;
      for (int d = 0; d < 3 && e == cudaSuccess; d++) {
        e = cudaMemcpy(&uu[d], c->d_u[c->cur][d] + slot, 4, cudaMemcpyDeviceToHost);
        if (e == cudaSuccess) e = cudaMemcpy(&vv[d], c->d_v[c->cur][d] + slot, 4, cudaMemcpyDeviceToHost);
      }
      if (e == cudaSuccess) e = cudaMemcpy(&spv, c->d_sp[c->cur] + slot, 1, cudaMemcpyDeviceToHost);
      if (e == cudaSuccess && c->has_wcorr) e = cudaMemcpy(&wcv, c->d_wc[c->cur] + slot, 4, cudaMemcpyDeviceToHost);
      s = cuda_check(c, e, "restart: last record");
      if (!s) {
        const int b = (int)(last_cell / AMPS_CPB);
        double x[3], vd[3], w = (double)wcv;
        for (int d = 0; d < 3; d++) {
          x[d] = origin[(size_t)(3 * b + d)] + (double)uu[d] * bdx[(size_t)(3 * b + d)];
          vd[d] = (double)vv[d];
        }
        std::memset(last, 0, sizeof(last));
        std::memcpy(last + L.off_v, vd, 24);
        std::memcpy(last + L.off_x, x, 24);
        last[L.off_sp] = spv;
        if (L.off_w >= 0) std::memcpy(last + L.off_w, &w, 8);
        // the 64-bit accumulator of the reference over the last record
        unsigned long long a64 = acc;
        for (int q = 0; q < L.len; q++) {
          const int i = (int)(((a64 >> 24) ^ last[q]) & 0xffull);
          a64 = (a64 << 8) ^ t64[i];
        }
        *checksum = a64;
      }
    }
  }
  cudaFree(d_crc);
  cudaFree(d_chunk);
  cudaFree(d_m);
  return s;
}

amps_gpu_status amps_gpu_read_restart_particles(amps_gpu_ctx* c, const amps_gpu_record_layout* layout,
                                                const void* data, long long size, const void* node_ids,
                                                int id_length, long long* nread) {
  if (!c || !layout || !data || size < 0 || id_length < 0 || (id_length > 0 && !node_ids))
    return AMPS_GPU_INVALID_ARG;
  const Layout L = layout_of(layout);
  if (!layout_ok(L)) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: bad record layout");
  const uint8_t* in = static_cast<const uint8_t*>(data);
  const long long header = kMarkerLen + 8 + 8LL * c->cfg.nspec;
  if (size < header || std::memcmp(in, kMarker, kMarkerLen) != 0)
    return set_err(c, AMPS_GPU_INVALID_ARG, "restart: the particle section marker is missing");
  long long len = 0;
  std::memcpy(&len, in + kMarkerLen, 8);
  if (len != L.len) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: ParticleDataLength differs from the layout");
  double weight[AMPS_GPU_MAX_SPECIES];
  std::memcpy(weight, in + kMarkerLen + 8, 8 * (size_t)c->cfg.nspec);
  // node id -> block
  std::unordered_map<std::string, int> block_of;
  for (int b = 0; b < c->nb; b++) {
    const char* idb = static_cast<const char*>(node_ids) + (size_t)b * id_length;
    if (!block_of.emplace(std::string(idb, (size_t)id_length), b).second)
      return set_err(c, AMPS_GPU_INVALID_ARG, "restart: node ids are not unique");
  }
  const long long ncell = c->ncor;
  std::vector<int> cnt((size_t)ncell, 0);
  std::vector<long long> cell_byte((size_t)ncell, 0), cell_rec((size_t)ncell, 0);
  std::vector<char> seen((size_t)c->nb, 0);
  long long pos = header, rec = 0;
  const long long bh = id_length + 4 + 4LL * AMPS_CPB;
  while (pos < size) {
    if (size - pos < bh) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: truncated block header");
    const auto it = block_of.find(std::string(reinterpret_cast<const char*>(in + pos), (size_t)id_length));
    if (it == block_of.end()) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: unknown node id");
    const int b = it->second;
    if (seen[(size_t)b]) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: block stored twice");
    seen[(size_t)b] = 1;
    int tot = 0;
    int table[AMPS_CPB];
    std::memcpy(&tot, in + pos + id_length, 4);
    std::memcpy(table, in + pos + id_length + 4, sizeof(table));
    pos += bh;
    long long sum = 0;
    for (int i = 0; i < 8; i++)
      for (int j = 0; j < 8; j++)
        for (int k = 0; k < 8; k++) {
          const int n = table[i * 64 + j * 8 + k];
          if (n < 0) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: negative cell count");
          const long long cid = (long long)b * AMPS_CPB + i + 8 * (j + 8 * k);
          cnt[(size_t)cid] = n;
          cell_byte[(size_t)cid] = pos;
          cell_rec[(size_t)cid] = rec;
          pos += (long long)n * L.len;
          rec += n;
          sum += n;
        }
    if (sum != tot) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: block count differs from its cell table");
    if (pos > size) return set_err(c, AMPS_GPU_INVALID_ARG, "restart: truncated particle records");
  }
  if (rec > c->cap) return set_err(c, AMPS_GPU_CAPACITY_EXCEEDED, "restart: more particles than the capacity");
  cudaSetDevice(c->cfg.device);
  std::vector<double> origin, bdx;
  block_geometry(c, origin, bdx);
  const bool wc = L.off_w >= 0;
  cudaError_t e = cudaSuccess;
  // page-locked input is read in place by the device, else copied in one transfer
  const uint8_t* direct = static_cast<const uint8_t*>(mapped_ptr(in));
  uint8_t* d_in = nullptr;
  unsigned long long* d_bad = nullptr;
  if (!direct) {
    e = cudaMalloc(reinterpret_cast<void**>(&d_in), (size_t)std::max<long long>(size, 1));
    if (e == cudaSuccess) e = cudaMemcpy(d_in, in, (size_t)size, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&d_bad), 2 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, 2 * sizeof(unsigned long long), c->stream);
  double* d_origin = dev_upload(origin, e);
  double* d_bdx = dev_upload(bdx, e);
  long long* d_byte = dev_upload(cell_byte, e);
  long long* d_rec = dev_upload(cell_rec, e);
  if (e == cudaSuccess) e = cudaMemcpy(c->d_count, cnt.data(), sizeof(int) * ncell, cudaMemcpyHostToDevice);
  unsigned long long bad[2] = {0, 0};
  if (e == cudaSuccess) {
    c->has_wcorr = wc;
    const int o = c->cur ^ 1;
    UnpackArgs a{};
    a.in = direct ? direct : d_in;
    a.cnt = c->d_count;
    a.cell_byte = d_byte;
    a.cell_rec = d_rec;
    a.origin = d_origin;
    a.bdx = d_bdx;
    a.ncell = ncell;
    a.L = L;
    a.nspec = c->cfg.nspec;
    for (int d = 0; d < 3; d++) {
      a.u[d] = c->d_u[o][d];
      a.v[d] = c->d_v[o][d];
    }
    a.sp = c->d_sp[o];
    a.wc = wc ? c->d_wc[o] : nullptr;
    a.id = c->cfg.track_ids ? c->d_id[o] : nullptr;
    a.key = c->d_key;
    a.rank = c->d_rank;
    a.bad = d_bad;
    const int wpb = kUnpackThreads / 32;
    const long long blocks = std::max<long long>(1, std::min<long long>((ncell + wpb - 1) / wpb, 152LL * 32));
    k_unpack<<<(unsigned)blocks, kUnpackThreads, (size_t)wpb * 32 * L.len, c->stream>>>(a);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = place_ranked(c, rec);
    if (e == cudaSuccess) e = cudaMemcpyAsync(bad, d_bad, sizeof(bad), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  }
  cudaFree(d_in);
  cudaFree(d_bad);
  cudaFree(d_origin);
  cudaFree(d_bdx);
  cudaFree(d_byte);
  cudaFree(d_rec);
  amps_gpu_status s = cuda_check(c, e, "restart: read");
  if (s) return s;
  c->np = rec;
  set_next_id(c, rec);
  c->have_moments = false;
  for (int q = 0; q < c->cfg.nspec; q++) c->cfg.weight[q] = weight[q];
  if (nread) *nread = rec;
  if (bad[0] || bad[1])
    return set_err(c, AMPS_GPU_INVALID_ARG,
                   "restart: " + std::to_string(bad[0]) + " records outside their cell, " +
                       std::to_string(bad[1]) + " with an unknown species (kept, clamped)");
  return AMPS_GPU_OK;
}

}  // extern "C"
