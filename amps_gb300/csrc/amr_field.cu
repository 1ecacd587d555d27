// ECSIM field kernels on block-structured AMR meshes (FP64), and the AMR
// variants of the particle import/export and stencil packing.
//
// The operator is assembled per cell in weak form (each term times the cell
// volume V): identity/8, (theta c dt)^2 C^T C with C the face-average curl of
// UpdateB (pic_field_solver_ecsim.cpp:5160-5711) whose transpose is the curl B
// of the RHS supports (src/pic/ecsim/get_stencil.cpp:1500-1599), and
// 4 pi theta dt M from the per-cell mass-matrix partials of ProcessCell
// (:1882-2438).  Corners of fine blocks that lie on a coarser block's face or
// edge off its corner lattice are hanging: they take the interpolation of the
// coarse corners (P), contributions to them are scattered to the parents (P^T),
// and their rows read x_h - (P x)_h = 0.  On a uniform mesh this is the
// reference operator times V.  One thread per cell, FP64 atomics for the
// scatter to the (up to 8) cells sharing a corner.
#include <cuda_runtime.h>

#include <algorithm>

#include "common.cuh"
#include "deposit_core.cuh"

namespace {

constexpr double kPi = 3.14159265358979323846264338327950288;
__constant__ int c_off[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

struct Hang {
  const int* hs;
  const int* hp;
  const double* hw;
  const float* hwh;  // hw as FP32 pairs
  const float* hwl;
  // boundary rows of meshes with open axes (bflag null: none): row b reads
  // x_b - sum_{t in [bs[b], bs[b+1])} bw[t] x_{bc[t]}
  const int* bflag;
  const int* bs;
  const int* bc;
  const double* bw;
  const float* bwh;
  const float* bwl;
};
__device__ __forceinline__ bool is_bnd(const Hang& h, long long c) { return h.bflag && h.bflag[c]; }

// value of corner c of a component-major field (component d), P applied,
// optionally scaled by a diagonal (right preconditioner)
__device__ __forceinline__ double cval(const double* __restrict__ F, const double* __restrict__ dinv,
                                       long long nvc, int c, int d, const Hang& h) {
  const int s = h.hs[c], e = h.hs[c + 1];
  if (s == e) return dinv ? dinv[d * nvc + c] * F[d * nvc + c] : F[d * nvc + c];
  double v = 0.0;
  for (int t = s; t < e; t++) {
    const int p = h.hp[t];
    v += h.hw[t] * (dinv ? dinv[d * nvc + p] * F[d * nvc + p] : F[d * nvc + p]);
  }
  return v;
}

// FP32 value of corner c, component d (xf already scaled), P applied
__device__ __forceinline__ float cval_f(const float* __restrict__ xf, long long nvc, int c, int d,
                                        const Hang& h) {
  // the value is loaded alongside the hanging test (one dependent load fewer)
  const float v0 = xf[d * nvc + c];
  const int s = h.hs[c], e = h.hs[c + 1];
  if (s == e) return v0;
  float v = 0.f;
  for (int t = s; t < e; t++) v = fmaf(h.hwh[t], xf[d * nvc + h.hp[t]], v);
  return v;
}

// corner c, component d of a field given as FP32 pairs (xh + xl), P applied in pairs
__device__ __forceinline__ FF cval_ff(const float* __restrict__ xh, const float* __restrict__ xl,
                                     long long nvc, int c, int d, const Hang& h) {
  const FF v0{xh[d * nvc + c], xl[d * nvc + c]};
  const int s = h.hs[c], e = h.hs[c + 1];
  if (s == e) return v0;
  FF v{0.f, 0.f};
  for (int t = s; t < e; t++) {
    const long long q = d * nvc + h.hp[t];
    ff_add2(v, h.hwh[t], h.hwl[t], xh[q], xl[q]);
  }
  return ff_norm(v);
}

// scatter out[8][3] to the cell's corners with P^T
template <typename T>
__device__ __forceinline__ void scatter(T* __restrict__ y, long long nvc, const int cid[8],
                                        const T out[8][3], const Hang& h) {
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int cc = cid[c], s = h.hs[cc], e = h.hs[cc + 1];
    if (s == e) {
#pragma unroll
      for (int d = 0; d < 3; d++) atomicAdd(y + d * nvc + cc, out[c][d]);
    } else {
      for (int t = s; t < e; t++) {
        const T w = (T)h.hw[t];
#pragma unroll
        for (int d = 0; d < 3; d++) atomicAdd(y + d * nvc + h.hp[t], w * out[c][d]);
      }
    }
  }
}

template <typename T>
__device__ __forceinline__ void cell_curl(const T e[8][3], T q, T cu[3]) {
  T a = 0, b = 0, c = 0, d = 0, f = 0, g = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const bool px = k == 1 || k == 2 || k == 5 || k == 6;
    const bool py = k == 2 || k == 3 || k == 6 || k == 7;
    const bool pz = k >= 4;
    a += py ? e[k][2] : -e[k][2];
    b += pz ? e[k][1] : -e[k][1];
    c += pz ? e[k][0] : -e[k][0];
    d += px ? e[k][2] : -e[k][2];
    f += px ? e[k][1] : -e[k][1];
    g += py ? e[k][0] : -e[k][0];
  }
  cu[0] = q * (a - b);
  cu[1] = q * (c - d);
  cu[2] = q * (f - g);
}

// out += s C^T y  (C with the 1/(4 dx) factor folded into s)
template <typename T>
__device__ __forceinline__ void cell_curl_t(const T y[3], T s, T out[8][3]) {
  const T a0 = s * y[0], a1 = s * y[1], a2 = s * y[2];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const bool px = k == 1 || k == 2 || k == 5 || k == 6;
    const bool py = k == 2 || k == 3 || k == 6 || k == 7;
    const bool pz = k >= 4;
    out[k][0] += (pz ? a1 : -a1) - (py ? a2 : -a2);
    out[k][1] += (px ? a2 : -a2) - (pz ? a0 : -a0);
    out[k][2] += (py ? a0 : -a0) - (px ? a1 : -a1);
  }
}

// out[k] += component p of s C^T y on the 8 corners
template <typename T>
__device__ __forceinline__ void cell_curl_t_row(const T y[3], T s, int p, T out[8]) {
  const T a0 = s * y[0], a1 = s * y[1], a2 = s * y[2];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const bool px = k == 1 || k == 2 || k == 5 || k == 6;
    const bool py = k == 2 || k == 3 || k == 6 || k == 7;
    const bool pz = k >= 4;
    if (p == 0) out[k] += (pz ? a1 : -a1) - (py ? a2 : -a2);
    else if (p == 1) out[k] += (px ? a2 : -a2) - (pz ? a0 : -a0);
    else out[k] += (py ? a0 : -a0) - (px ? a1 : -a1);
  }
}

// scatter component p of out[8] to the cell's corners with P^T
template <typename T>
__device__ __forceinline__ void scatter_row(T* __restrict__ y, long long nvc, const int cid[8], int p,
                                            const T out[8], const Hang& h) {
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int cc = cid[c], s = h.hs[cc], e = h.hs[cc + 1];
    if (s == e) {
      atomicAdd(y + p * nvc + cc, out[c]);
    } else {
      for (int t = s; t < e; t++) atomicAdd(y + p * nvc + h.hp[t], (T)h.hw[t] * out[c]);
    }
  }
}

// per cell size (index log2 of the block's cell size in finest cells): the
// operator's scale factors, FP32 for the inner operator and as FP32 pairs
struct LevelK {
  float dx, V;                       // FP32 inner operator
  float curl[2], cc[2], id[2], m[2], bb[2];  // 0.25/dx, th2dt2 V 0.25/dx, V/8, f V, thdt V 0.25/dx
};
constexpr int kMaxScale = 8;

struct ApplyArgs {
  long long ncell, nvc;
  const int* ctab;
  Hang h;
  const int* bscale;
  LevelK lk[kMaxScale];
  float fj[2];          // f as a pair (the current term of the RHS)
  const float* xh;      // ACC 1/2 input as FP32 pairs (dinv applied)
  const float* xl;
  const double* bdx;
  const float* cellM;
  const float* cellJ;
  const double* x;     // input field (component-major)
  const float* xf;     // the same times dinv, in FP32 (the FP32 inner operator)
  const double* dinv;  // optional right preconditioner
  const double* Bcen;  // RHS: centre B (component-major over cells)
  double th2dt2, f, thdt;
  unsigned long long* flags;  // [2]: bounded-wait timeouts
};

// ---------------------------------------------------------------------------
// The operator per cell (weak form, see above), y += its contributions.  A CTA
// serves 32 cells with 3 threads each (one per output component p; warp p
// takes the 32 cells): the cells' run of partials (31,104 contiguous bytes) is
// brought into shared memory by one bulk copy while the threads gather the
// corner values (each value once, shared through shared memory), and each
// thread reads the rows 3p..3p+2 of its cell's 27 monomial blocks from there
// (stride 243 words between a warp's cells: conflict-free).
//   ACC 0: FP32 inner operator (curl-curl + mass; identity added in FP64 by
//          k_amr_finish32), FP32 atomics;
//   ACC 1: the full operator to FP64 accuracy (outer residuals);
//   ACC 2: the RHS to FP64 accuracy.
// ACC 1/2 run in FP32 pairs (FF, common.cuh): FP64 arithmetic is a small
// fraction of the FP32 rate on this part; the pairs carry FP64 accuracy.
constexpr int kTileCells = 32;
constexpr int kTileThreads = 3 * kTileCells;
constexpr uint32_t kTileBytes = kTileCells * AMPS_CELLM * 4;  // 31,104

template <int ACC>
__global__ void __launch_bounds__(kTileThreads) k_amr_cell_tile(ApplyArgs a, float* __restrict__ y32,
                                                               double* __restrict__ y64) {
  extern __shared__ __align__(16) float s_m[];
  __shared__ __align__(8) uint64_t bar;
  // corner values (8 corners x 3): FP32 for ACC 0, FP32 pairs for ACC 1/2
  __shared__ float s_eh[kTileCells][24];
  __shared__ float s_el[ACC == 0 ? 1 : kTileCells][24];
  // the cell's curl (and for the RHS its centre B) as pairs, one component per thread
  __shared__ float s_cu[ACC == 0 ? 1 : kTileCells][3][2];
  __shared__ float s_b[ACC == 2 ? kTileCells : 1][3][2];
  // ACC 0: the tile's 32 cells (an 8 x 4 x 1 slab of a block) share 9 x 5 x 2
  // corners; their contributions are summed in shared memory first, so each
  // corner gets one global atomic per component instead of up to 8
  constexpr int kTC = 90;
  __shared__ float s_acc[ACC == 0 ? 3 * kTC : 1];
  __shared__ int s_tcid[kTC];
  // ACC 1/2: the same per-corner sums as pairs, accumulated without atomics:
  // warp p owns component p, and in round c the 32 cells' corner c are 32
  // distinct tile corners
  __shared__ float s_ffacc[ACC == 0 ? 1 : 3][ACC == 0 ? 1 : kTC][2];
  const int tid = threadIdx.x, p = tid / kTileCells, lc = tid % kTileCells;
  const long long cell0 = (long long)blockIdx.x * kTileCells;
  if (tid == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    mbar_arrive_expect_tx(&bar, kTileBytes);
    bulk_copy_g2s(s_m, a.cellM + cell0 * AMPS_CELLM, kTileBytes, &bar);
  }
  const long long cell = cell0 + lc;
  const int b = (int)(cell >> 9), l = (int)(cell & 511);
  const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
  const LevelK& K = a.lk[min(__ffs(a.bscale[b]) - 1, kMaxScale - 1)];
  // the cell's corners and their values, each gathered once by one of its 3
  // threads (thread p: corner ids c = p, p+3, p+6; values of component p)
  // tile-local corner of (cell lc, corner c): the slab's cells are i = 0..7,
  // 4 rows j, one k
  auto tcorner = [&](int c) { return (lc % 8 + c_off[c][0]) + 9 * ((lc / 8 + c_off[c][1]) + 5 * c_off[c][2]); };
  // every thread loads its cell's 8 corner ids (cached table), so the value
  // gathers below wait on one load, not on a barrier
  int cid[8];
#pragma unroll
  for (int c = 0; c < 8; c++) {
    cid[c] = a.ctab[b * 729 + (i + c_off[c][0]) + 9 * ((j + c_off[c][1]) + 9 * (k + c_off[c][2]))];
    if (c % 3 == p) s_tcid[tcorner(c)] = cid[c];  // the same id from every cell sharing it
  }
  if (ACC == 0) {
    for (int q = tid; q < 3 * kTC; q += kTileThreads) s_acc[q] = 0.f;
  } else {
    for (int q = tid; q < 3 * kTC; q += kTileThreads) {
      s_ffacc[q / kTC][q % kTC][0] = 0.f;
      s_ffacc[q / kTC][q % kTC][1] = 0.f;
    }
  }
  if (ACC == 2) {
    // centre B, component p, split into a pair (the only FP64 arithmetic besides the scatter)
    const double Bv = a.Bcen[p * a.ncell + cell];
    const float bh = (float)Bv;
    s_b[lc][p][0] = bh;
    s_b[lc][p][1] = (float)(Bv - (double)bh);
  }
#pragma unroll
  for (int c = 0; c < 8; c++) {
    if (ACC == 0) {
      s_eh[lc][3 * c + p] = cval_f(a.xf, a.nvc, cid[c], p, a.h);
    } else {
      const FF v = cval_ff(a.xh, a.xl, a.nvc, cid[c], p, a.h);
      s_eh[lc][3 * c + p] = v.s;
      s_el[lc][3 * c + p] = v.q;
    }
  }
  // CTA-uniform: every thread leaves together on a timeout (later barriers)
  const bool ok = __syncthreads_and(mbar_wait_bounded(&bar, 0, kWaitLimit)) != 0;
  if (!ok) {
    if (tid == 0) atomicAdd(a.flags + 2, 1ull);
    mbar_wait_bounded(&bar, 0, kWaitLimit);  // let the copy land before exiting
    return;
  }
  const float* mm = s_m + lc * AMPS_CELLM + 3 * p;  // row p of every monomial block
  if (ACC == 0) {
    const float dx = K.dx, V = K.V;
    float ef[8][3], out[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      out[c] = 0.f;
#pragma unroll
      for (int d = 0; d < 3; d++) ef[c][d] = s_eh[lc][3 * c + d];
    }
    float cu[3];
    cell_curl<float>(ef, 0.25f / dx, cu);
    cell_curl_t_row<float>(cu, (float)a.th2dt2 * V * 0.25f / dx, p, out);
    const float fv = (float)a.f * V;
#pragma unroll
    for (int c1 = 0; c1 < 8; c1++)
#pragma unroll
      for (int c2 = 0; c2 <= c1; c2++) {
        const float* m3 = mm + pair_monomial(c1, c2) * 9;
        const float m0 = fv * m3[0], m1 = fv * m3[1], m2 = fv * m3[2];
        out[c1] += m0 * ef[c2][0] + m1 * ef[c2][1] + m2 * ef[c2][2];
        if (c1 != c2) out[c2] += m0 * ef[c1][0] + m1 * ef[c1][1] + m2 * ef[c1][2];
      }
#pragma unroll
    for (int c = 0; c < 8; c++) atomicAdd(&s_acc[3 * tcorner(c) + p], out[c]);
    __syncthreads();
    // one global atomic per tile corner and component (P^T for hanging corners)
    for (int q = tid; q < 3 * kTC; q += kTileThreads) {
      const int tc = q / 3, pp = q % 3, cc = s_tcid[tc];
      const float v = s_acc[q];
      const int hs0 = a.h.hs[cc], hs1 = a.h.hs[cc + 1];
      if (hs0 == hs1) {
        atomicAdd(y32 + pp * a.nvc + cc, v);
      } else {
        for (int t = hs0; t < hs1; t++) atomicAdd(y32 + pp * a.nvc + a.h.hp[t], a.h.hwh[t] * v);
      }
    }
  } else {
    const float sg = ACC == 2 ? -1.f : 1.f;
    FF out[8];
#pragma unroll
    for (int c = 0; c < 8; c++)
      out[c] = ACC == 1 ? ff_mul(s_eh[lc][3 * c + p], s_el[lc][3 * c + p], K.id[0], K.id[1]) : FF{0.f, 0.f};
    // the curl's component p: cu_p = 0.25/dx (sum +-E_qa - sum +-E_qb)
    const int qa = p == 0 ? 2 : (p == 1 ? 0 : 1), qb = p == 0 ? 1 : (p == 1 ? 2 : 0);
    {
      FF d{0.f, 0.f};
#pragma unroll
      for (int k2 = 0; k2 < 8; k2++) {
        const bool px = k2 == 1 || k2 == 2 || k2 == 5 || k2 == 6;
        const bool py = k2 == 2 || k2 == 3 || k2 == 6 || k2 == 7;
        const bool pz = k2 >= 4;
        // cu0 = (dEz/dy - dEy/dz), cu1 = (dEx/dz - dEz/dx), cu2 = (dEy/dx - dEx/dy)
        const bool sga = p == 0 ? py : (p == 1 ? pz : px);
        const bool sgb = p == 0 ? pz : (p == 1 ? px : py);
        const float ha = s_eh[lc][3 * k2 + qa], la = s_el[lc][3 * k2 + qa];
        const float hb = s_eh[lc][3 * k2 + qb], lb = s_el[lc][3 * k2 + qb];
        ff_acc(d, sga ? ha : -ha, sga ? la : -la);
        ff_acc(d, sgb ? -hb : hb, sgb ? -lb : lb);
      }
      d = ff_norm(d);
      const FF cu = ff_norm(ff_mul(d.s, d.q, K.curl[0], K.curl[1]));
      s_cu[lc][p][0] = cu.s;
      s_cu[lc][p][1] = cu.q;
    }
    __syncthreads();
    // out[k] += s (sig1 y[q1] - sig2 y[q2]) for y = the curl (s = sg th2dt2 V 0.25/dx)
    // and, for the RHS, y = centre B (s = thdt V 0.25/dx): C^T y, component p
    const int q1 = p == 0 ? 1 : (p == 1 ? 2 : 0), q2 = p == 0 ? 2 : (p == 1 ? 0 : 1);
    auto curl_t = [&](float (*y)[2], float sh, float sl) {
      FF tpp{y[q1][0], y[q1][1]}, tpm{y[q1][0], y[q1][1]};
      ff_acc(tpp, -y[q2][0], -y[q2][1]);  // y1 - y2
      ff_acc(tpm, y[q2][0], y[q2][1]);    // y1 + y2
      tpp = ff_norm(tpp);
      tpm = ff_norm(tpm);
      const FF upp = ff_mul(tpp.s, tpp.q, sh, sl), upm = ff_mul(tpm.s, tpm.q, sh, sl);
#pragma unroll
      for (int k2 = 0; k2 < 8; k2++) {
        const bool px = k2 == 1 || k2 == 2 || k2 == 5 || k2 == 6;
        const bool py = k2 == 2 || k2 == 3 || k2 == 6 || k2 == 7;
        const bool pz = k2 >= 4;
        const bool s1 = p == 0 ? pz : (p == 1 ? px : py);
        const bool s2 = p == 0 ? py : (p == 1 ? pz : px);
        // s1 y1 - s2 y2: (+,+) y1 - y2, (+,-) y1 + y2, (-,+) -(y1 + y2), (-,-) -(y1 - y2)
        const FF& u = (s1 == s2) ? upp : upm;
        const float sgn = s1 ? 1.f : -1.f;
        ff_acc(out[k2], sgn * u.s, sgn * u.q);
      }
    };
    curl_t(s_cu[lc], sg * K.cc[0], sg * K.cc[1]);
    // mass term: sum over pairs of m (FP32 partial) x e, in FP32 pairs
    float eh[8][3], el[8][3];
    FF acc[8];
#pragma unroll
    for (int c = 0; c < 8; c++) {
      acc[c] = FF{0.f, 0.f};
#pragma unroll
      for (int d = 0; d < 3; d++) {
        eh[c][d] = s_eh[lc][3 * c + d];
        el[c][d] = s_el[lc][3 * c + d];
      }
    }
#pragma unroll
    for (int c1 = 0; c1 < 8; c1++)
#pragma unroll
      for (int c2 = 0; c2 <= c1; c2++) {
        const float* m3 = mm + pair_monomial(c1, c2) * 9;
#pragma unroll
        for (int q = 0; q < 3; q++) {
          const float m = m3[q];
          ff_add(acc[c1], m, eh[c2][q], el[c2][q]);
          if (c1 != c2) ff_add(acc[c2], m, eh[c1][q], el[c1][q]);
        }
      }
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const FF t = ff_norm(acc[c]);
      const FF u = ff_mul(t.s, t.q, sg * K.m[0], sg * K.m[1]);
      ff_acc(out[c], u.s, u.q);
    }
    if (ACC == 2) {
      curl_t(s_b[lc], K.bb[0], K.bb[1]);
      const float* jj = a.cellJ + cell * 24;
#pragma unroll
      for (int c = 0; c < 8; c++) ff_add2(out[c], -a.fj[0], -a.fj[1], jj[3 * c + p], 0.f);
    }
    // sum over the tile's cells per corner, in pairs (round c: corner c of every cell)
#pragma unroll
    for (int c = 0; c < 8; c++) {
      float* slot = s_ffacc[p][tcorner(c)];
      FF v{slot[0], slot[1]};
      ff_acc(v, out[c].s, out[c].q);
      slot[0] = v.s;
      slot[1] = v.q;
      __syncwarp();
    }
    __syncthreads();
    // scatter with P^T: one FP64 atomic per tile corner and component
    for (int q = tid; q < 3 * kTC; q += kTileThreads) {
      const int pp = q / kTC, tc = q % kTC, cc = s_tcid[tc];
      const FF o = ff_norm(FF{s_ffacc[pp][tc][0], s_ffacc[pp][tc][1]});
      const int hs0 = a.h.hs[cc], hs1 = a.h.hs[cc + 1];
      if (hs0 == hs1) {
        atomicAdd(y64 + pp * a.nvc + cc, ff_value(o));
      } else {
        for (int t = hs0; t < hs1; t++)
          atomicAdd(y64 + pp * a.nvc + a.h.hp[t], ff_value(ff_mul(o.s, o.q, a.h.hwh[t], a.h.hwl[t])));
      }
    }
  }
}

// x (times dinv) as FP32 pairs: the input of the pair-arithmetic operator
__global__ void __launch_bounds__(256) k_amr_split(long long n, const double* __restrict__ x,
                                                   const double* __restrict__ dinv,
                                                   float* __restrict__ xh, float* __restrict__ xl) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x) {
    const double v = dinv ? dinv[t] * x[t] : x[t];
    const float h = (float)v;
    xh[t] = h;
    xl[t] = (float)(v - (double)h);
  }
}

// xf = fp32(dinv .* x), the FP32 inner operator's input
__global__ void __launch_bounds__(256) k_amr_to_f32(long long n, const double* __restrict__ x,
                                                    const double* __restrict__ dinv,
                                                    float* __restrict__ xf) {
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long)gridDim.x * blockDim.x)
    xf[t] = (float)(dinv ? dinv[t] * x[t] : x[t]);
}

// The same with the input and output as FP32 pairs (Krylov vectors): free
// rows S (D v) + y32 in pairs, hanging rows (D v)_h - (P D v)_h.
__global__ void __launch_bounds__(256) k_amr_finish_ff(long long nvc, Hang h,
                                                       const int* __restrict__ ss,
                                                       const int* __restrict__ sc,
                                                       const float* __restrict__ svh,
                                                       const float* __restrict__ svl,
                                                       const float* __restrict__ y32, OpIn in,
                                                       float* __restrict__ wh, float* __restrict__ wl) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nvc) return;
  int s = h.hs[c], e = h.hs[c + 1];
  const int* col = h.hp;
  const float* cwh = h.hwh;
  const float* cwl = h.hwl;
  const bool bnd = s == e && is_bnd(h, c);
  if (bnd) {
    s = h.bs[c];
    e = h.bs[c + 1];
    col = h.bc;
    cwh = h.bwh;
    cwl = h.bwl;
  }
#pragma unroll
  for (int d = 0; d < 3; d++) {
    FF acc;
    if (s == e && !bnd) {
      acc = FF{y32[d * nvc + c], 0.f};
      for (int q = ss[c]; q < ss[c + 1]; q++) {
        const FF v = opin_value(in, d * nvc + sc[q]);
        ff_add2(acc, svh[q], svl[q], v.s, v.q);
      }
    } else {
      // constraint rows: hanging (parents) or boundary (donors)
      acc = opin_value(in, d * nvc + c);
      for (int t = s; t < e; t++) {
        const FF v = opin_value(in, d * nvc + col[t]);
        ff_add2(acc, -cwh[t], -cwl[t], v.s, v.q);
      }
    }
    acc = ff_norm(acc);
    wh[d * nvc + c] = acc.s;
    wl[d * nvc + c] = acc.q;
  }
}

// Free rows: the identity part S (D x) in FP64 (S = P^T diag(sum of V/8) P,
// mostly diagonal, CSR) plus the FP32 accumulation of the other terms.
// Hanging rows: the constraint x_h - (P x)_h in FP64.
__global__ void __launch_bounds__(256) k_amr_finish32(long long nvc, Hang h,
                                                      const int* __restrict__ ss,
                                                      const int* __restrict__ sc,
                                                      const double* __restrict__ sv,
                                                      const float* __restrict__ y32,
                                                      const double* __restrict__ x,
                                                      const double* __restrict__ dinv,
                                                      double* __restrict__ y) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nvc) return;
  int s = h.hs[c], e = h.hs[c + 1];
  const int* col = h.hp;
  const double* w = h.hw;
  const bool bnd = s == e && is_bnd(h, c);
  if (bnd) {
    s = h.bs[c];
    e = h.bs[c + 1];
    col = h.bc;
    w = h.bw;
  }
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (s == e && !bnd) {
      double acc = (double)y32[d * nvc + c];
      for (int q = ss[c]; q < ss[c + 1]; q++) {
        const int cl = sc[q];
        acc += sv[q] * (dinv ? dinv[d * nvc + cl] : 1.0) * x[d * nvc + cl];
      }
      y[d * nvc + c] = acc;
    } else {
      // constraint rows: hanging (parents) or boundary (donors)
      double pv = 0.0;
      for (int t = s; t < e; t++) {
        const int p = col[t];
        pv += w[t] * (dinv ? dinv[d * nvc + p] : 1.0) * x[d * nvc + p];
      }
      y[d * nvc + c] = (dinv ? dinv[d * nvc + c] : 1.0) * x[d * nvc + c] - pv;
    }
  }
}

// hanging rows: y_h = x_h - (P x)_h (operator) or 0 (rhs)
__global__ void __launch_bounds__(256) k_amr_constraint(long long nvc, Hang h,
                                                        const double* __restrict__ x,
                                                        const double* __restrict__ dinv,
                                                        double* __restrict__ y, int rhs_mode) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nvc) return;
  int s = h.hs[c], e = h.hs[c + 1];
  const int* col = h.hp;
  const double* w = h.hw;
  if (s == e) {
    // boundary rows (open axes): the same form with the donor list
    if (!is_bnd(h, c)) return;
    s = h.bs[c];
    e = h.bs[c + 1];
    col = h.bc;
    w = h.bw;
  }
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (rhs_mode) {
      y[d * nvc + c] = 0.0;
    } else {
      double pv = 0.0;
      for (int t = s; t < e; t++) {
        const int p = col[t];
        pv += w[t] * (dinv ? dinv[d * nvc + p] : 1.0) * x[d * nvc + p];
      }
      y[d * nvc + c] = (dinv ? dinv[d * nvc + c] : 1.0) * x[d * nvc + c] - pv;
    }
  }
}

// Jacobi diagonal (free corners: sum over their cells of the cell diagonal)
// Jacobi diagonal (a preconditioner: FP32 arithmetic is enough; per cell size
// s: base[s] = V (1/8 + th2dt2 / (8 dx^2)), fv[s] = f V)
struct DiagK {
  float base[kMaxScale], fv[kMaxScale];
};
__global__ void __launch_bounds__(256) k_amr_diag(long long ncell, long long nvc, const int* ctab,
                                                  Hang h, const int* bscale, const float* cellM, DiagK K,
                                                  double* diag) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncell) return;
  const int b = (int)(cell >> 9), l = (int)(cell & 511);
  const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
  const int sc = min(__ffs(bscale[b]) - 1, kMaxScale - 1);
  const float base = K.base[sc], fv = K.fv[sc];
  const float* mm = cellM + cell * AMPS_CELLM;
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int cc = ctab[b * 729 + (i + c_off[c][0]) + 9 * ((j + c_off[c][1]) + 9 * (k + c_off[c][2]))];
    const float* blk = mm + pair_monomial(c, c) * 9;
    const float m0 = blk[0], m1 = blk[4], m2 = blk[8];
    if (h.hs[cc + 1] > h.hs[cc]) continue;
    atomicAdd(diag + cc, (double)fmaf(fv, m0, base));
    atomicAdd(diag + nvc + cc, (double)fmaf(fv, m1, base));
    atomicAdd(diag + 2 * nvc + cc, (double)fmaf(fv, m2, base));
  }
}

__global__ void __launch_bounds__(256) k_amr_invert_diag(long long nvc, Hang h, double* diag) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nvc) return;
  const bool hang = h.hs[c + 1] > h.hs[c] || is_bnd(h, c);  // constraint rows: scaling 1
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const float v = (float)diag[d * nvc + c];  // a preconditioner: FP32 reciprocal
    diag[d * nvc + c] = (hang || v == 0.f) ? 1.0 : (double)(1.0f / v);
  }
}

__global__ void __launch_bounds__(256) k_amr_update_b(long long ncell, long long nvc,
                                                      const int* ctab, Hang h, const double* bdx,
                                                      const double* Eh, const double* Bn,
                                                      double* Bnew, double dt) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncell) return;
  const int b = (int)(cell >> 9), l = (int)(cell & 511);
  const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
  double e[8][3];
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int cc = ctab[b * 729 + (i + c_off[c][0]) + 9 * ((j + c_off[c][1]) + 9 * (k + c_off[c][2]))];
#pragma unroll
    for (int d = 0; d < 3; d++) e[c][d] = cval(Eh, nullptr, nvc, cc, d, h);
  }
  double cu[3];
  cell_curl<double>(e, 0.25 / bdx[b], cu);
#pragma unroll
  for (int d = 0; d < 3; d++) Bnew[d * ncell + cell] = Bn[d * ncell + cell] - dt * cu[d];
}

// UpdateB's boundary branch on meshes with open axes
// (pic_field_solver_ecsim.cpp:5274-5600): a cell with a face on an open domain
// face keeps B^n (Dirichlet, pass 0) or takes the mean of B^{n+1} of its
// face-normal inward neighbours, one per such face, in the same block
// (Neumann, pass p = number of such faces: faces, then edges, then corners, so
// every donor is final when read).  A cell on a Neumann face (bit 2d + high of
// neumann) is Neumann, whatever its other faces.
__global__ void __launch_bounds__(256) k_amr_bnd_b(long long ncell, const int* __restrict__ borg,
                                                   const int* __restrict__ bscale, int nf0, int nf1, int nf2,
                                                   int open, int neumann, int pass, const double* __restrict__ Bn,
                                                   double* __restrict__ Bnew) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncell) return;
  const int b = (int)(cell >> 9), l = (int)(cell & 511);
  const int idx[3] = {l & 7, (l >> 3) & 7, l >> 6};
  const int st = bscale[b], nf[3] = {nf0, nf1, nf2};
  int side[3] = {0, 0, 0}, nface = 0;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (!((open >> d) & 1)) continue;
    const int lo = borg[3 * b + d] + idx[d] * st;
    if (lo == 0) side[d] = -1;
    else if (lo + st == nf[d]) side[d] = 1;
    nface += side[d] != 0;
  }
  if (!nface) return;
  bool neu = false;
#pragma unroll
  for (int d = 0; d < 3; d++)
    if (side[d]) neu |= (neumann >> (2 * d + (side[d] > 0))) & 1;
  if (!neu) {
    if (pass == 0)
#pragma unroll
      for (int q = 0; q < 3; q++) Bnew[q * ncell + cell] = Bn[q * ncell + cell];
    return;
  }
  if (nface != pass) return;
  double acc[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (!side[d]) continue;
    int j[3] = {idx[0], idx[1], idx[2]};
    j[d] -= side[d];
    const long long dn = (long long)b * 512 + j[0] + 8 * (j[1] + 8 * j[2]);
#pragma unroll
    for (int q = 0; q < 3; q++) acc[q] += Bnew[q * ncell + dn];
  }
#pragma unroll
  for (int q = 0; q < 3; q++) Bnew[q * ncell + cell] = acc[q] / nface;
}

// C2N: accumulate V*B and V on the corners (P^T for hanging is not used: their
// value is re-interpolated afterwards)
__global__ void __launch_bounds__(256) k_amr_c2n_acc(long long ncell, long long nvc,
                                                     const int* ctab, const double* bdx,
                                                     const double* Bcen, double* acc,
                                                     double* wsum) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= ncell) return;
  const int b = (int)(cell >> 9), l = (int)(cell & 511);
  const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
  const double dx = bdx[b], V = dx * dx * dx;
  const double B[3] = {Bcen[cell], Bcen[ncell + cell], Bcen[2 * ncell + cell]};
#pragma unroll
  for (int c = 0; c < 8; c++) {
    const int cc = ctab[b * 729 + (i + c_off[c][0]) + 9 * ((j + c_off[c][1]) + 9 * (k + c_off[c][2]))];
    atomicAdd(wsum + cc, V);
#pragma unroll
    for (int d = 0; d < 3; d++) atomicAdd(acc + d * nvc + cc, V * B[d]);
  }
}

__global__ void __launch_bounds__(256) k_amr_c2n_div(long long nvc, const double* wsum,
                                                     double* acc) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nvc) return;
  const double w = wsum[c];
#pragma unroll
  for (int d = 0; d < 3; d++) acc[d * nvc + c] = w > 0.0 ? acc[d * nvc + c] / w : 0.0;
}

// hanging corners of a field take the interpolation of their (free) parents
__global__ void __launch_bounds__(256) k_amr_fix_hanging(long long nvc, Hang h, double* F) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nvc) return;
  const int s = h.hs[c], e = h.hs[c + 1];
  if (s == e) return;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    double v = 0.0;
    for (int t = s; t < e; t++) v += h.hw[t] * F[d * nvc + h.hp[t]];
    F[d * nvc + c] = v;
  }
}

__global__ void __launch_bounds__(256) k_amr_update_e(long long nvc, const double* Eh, double* En,
                                                      double theta) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nvc) return;
#pragma unroll
  for (int d = 0; d < 3; d++)
    En[d * nvc + c] = (Eh[d * nvc + c] - (1.0 - theta) * En[d * nvc + c]) / theta;
}

// wave energy sum_cells V (sum_corners |E|^2/8 + |B|^2) / (8 pi)
__global__ void __launch_bounds__(256) k_amr_wave_energy(long long ncell, long long nvc,
                                                         const int* ctab, const double* bdx,
                                                         const double* En, const double* Bcen,
                                                         double* energy) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double en = 0.0;
  if (cell < ncell) {
    const int b = (int)(cell >> 9), l = (int)(cell & 511);
    const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
    const double dx = bdx[b], V = dx * dx * dx;
    double e2 = 0.0;
#pragma unroll
    for (int c = 0; c < 8; c++) {
      const int cc = ctab[b * 729 + (i + c_off[c][0]) + 9 * ((j + c_off[c][1]) + 9 * (k + c_off[c][2]))];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const double v = En[d * nvc + cc];
        e2 += v * v;
      }
    }
    double b2 = 0.0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double v = Bcen[d * ncell + cell];
      b2 += v * v;
    }
    en = (0.125 * e2 + b2) * V * 0.125 / kPi;
  }
  __shared__ double s[8];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) en += __shfl_xor_sync(0xffffffffu, en, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = en;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s[w];
    atomicAdd(energy, t);
  }
}

__global__ void k_amr_pack(long long nvc, const int* ctab, Hang h, const double* Eh,
                           const double* Bprev, const double* Bcur, float* sp, float* sd) {
  const int b = blockIdx.x;
  for (int s = threadIdx.x; s < AMPS_SC; s += blockDim.x) {
    const int cc = ctab[b * 729 + s];
    float4* op = reinterpret_cast<float4*>(sp + ((size_t)b * AMPS_SC + s) * AMPS_PUSH_STRIDE);
    op[0] = make_float4((float)cval(Eh, nullptr, nvc, cc, 0, h), (float)cval(Eh, nullptr, nvc, cc, 1, h),
                        (float)cval(Eh, nullptr, nvc, cc, 2, h), (float)cval(Bprev, nullptr, nvc, cc, 0, h));
    op[1] = make_float4((float)cval(Bprev, nullptr, nvc, cc, 1, h),
                        (float)cval(Bprev, nullptr, nvc, cc, 2, h), 0.f, 0.f);
    reinterpret_cast<float4*>(sd)[(size_t)b * AMPS_SC + s] =
        make_float4((float)cval(Bcur, nullptr, nvc, cc, 0, h), (float)cval(Bcur, nullptr, nvc, cc, 1, h),
                    (float)cval(Bcur, nullptr, nvc, cc, 2, h), 0.f);
  }
}

Hang hang_of(const amps_gpu_ctx* c) {
  return Hang{c->d_hs, c->d_hp, c->d_hw, c->d_hwh, c->d_hwl,
              c->d_bflag, c->d_bs, c->d_bc, c->d_bw, c->d_bwh, c->d_bwl};
}
unsigned g1(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

// ============================================================================
cudaError_t launch_amr_pack(amps_gpu_ctx* c, const double* Eh, const double* Bprev,
                            const double* Bcur) {
  TimedLaunch t(c, "pack_stencils");
  k_amr_pack<<<c->nb, 256, 0, c->stream>>>(c->nvc, c->d_ctab, hang_of(c), Eh, Bprev, Bcur,
                                            c->d_stencil_push, c->d_stencil_dep);
  return cudaGetLastError();
}

static ApplyArgs apply_args(amps_gpu_ctx* c) {
  ApplyArgs a{};
  a.ncell = c->ncor;
  a.nvc = c->nvc;
  a.ctab = c->d_ctab;
  a.h = hang_of(c);
  a.bdx = c->d_bdx;
  a.cellM = c->d_cellM;
  a.cellJ = c->d_cellJ;
  const double th = c->cfg.theta, dt = c->cfg.dt;
  a.th2dt2 = th * th * dt * dt;
  a.f = 4.0 * kPi * dt * th;
  a.thdt = th * dt;
  a.flags = c->d_flags;
  a.bscale = c->d_bscale;
  auto split = [](double v, float* o) {
    o[0] = (float)v;
    o[1] = (float)(v - (double)o[0]);
  };
  for (int sc = 0; sc < kMaxScale; sc++) {
    const double dx = c->dxf * (double)(1 << sc), V = dx * dx * dx;
    LevelK& K = a.lk[sc];
    K.dx = (float)dx;
    K.V = (float)V;
    split(0.25 / dx, K.curl);
    split(a.th2dt2 * V * 0.25 / dx, K.cc);
    split(0.125 * V, K.id);
    split(a.f * V, K.m);
    split(a.thdt * V * 0.25 / dx, K.bb);
  }
  split(a.f, a.fj);
  return a;
}

// x (times dinv) as FP32 pairs in the context's scratch (2 x 3 nvc floats)
static cudaError_t split_input(amps_gpu_ctx* c, const double* x, const double* dinv, ApplyArgs& a) {
  const long long n = 3 * c->nvc;
  cudaError_t e = cudaSuccess;
  if (!c->d_xs && (e = cudaMalloc(reinterpret_cast<void**>(&c->d_xs), sizeof(float) * 2 * n)) != cudaSuccess)
    return e;
  a.xh = c->d_xs;
  a.xl = c->d_xs + n;
  k_amr_split<<<(unsigned)std::min<long long>((n + 255) / 256, 152LL * 16), 256, 0, c->stream>>>(n, x, dinv,
                                                                                                c->d_xs,
                                                                                                c->d_xs + n);
  return cudaGetLastError();
}

template <int ACC>
static cudaError_t launch_tile(amps_gpu_ctx* c, const ApplyArgs& a, float* y32, double* y64) {
  static unsigned long long attr_set = 0;  // per device
  int dev = 0;
  cudaGetDevice(&dev);
  if (!((attr_set >> dev) & 1ull)) {
    cudaError_t e = cudaFuncSetAttribute(k_amr_cell_tile<ACC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)kTileBytes);
    if (e != cudaSuccess) return e;
    attr_set |= 1ull << dev;
  }
  // AMR meshes hold whole 512-cell blocks: ncell is a multiple of the tile
  k_amr_cell_tile<ACC><<<(unsigned)(c->ncor / kTileCells), kTileThreads, kTileBytes, c->stream>>>(a, y32,
                                                                                                 y64);
  return cudaGetLastError();
}

cudaError_t launch_amr_matvec(amps_gpu_ctx* c, const double* x, const double* dinv, double* y) {
  cudaError_t e = cudaMemsetAsync(y, 0, sizeof(double) * 3 * c->nvc, c->stream);
  if (e != cudaSuccess) return e;
  ApplyArgs a = apply_args(c);
  a.x = x;
  a.dinv = dinv;
  TimedLaunch t(c, "matvec", 3);
  if ((e = split_input(c, x, dinv, a)) != cudaSuccess) return e;
  if ((e = launch_tile<1>(c, a, nullptr, y)) != cudaSuccess) return e;
  k_amr_constraint<<<g1(c->nvc), 256, 0, c->stream>>>(c->nvc, a.h, x, dinv, y, 0);
  return cudaGetLastError();
}

cudaError_t launch_amr_matvec32(amps_gpu_ctx* c, const double* x, const double* dinv,
                                double* y) {
  cudaError_t e = cudaMemsetAsync(c->d_y32, 0, sizeof(float) * 3 * c->nvc, c->stream);
  if (e != cudaSuccess) return e;
  ApplyArgs a = apply_args(c);
  a.x = x;
  a.dinv = dinv;
  // the identity part is applied in FP64 by k_amr_finish32
  const long long n = 3 * c->nvc;
  if (!c->d_xs && (e = cudaMalloc(reinterpret_cast<void**>(&c->d_xs), sizeof(float) * 2 * n)) != cudaSuccess)
    return e;
  a.xf = c->d_xs;
  TimedLaunch t(c, "matvec32", 3);
  k_amr_to_f32<<<(unsigned)std::min<long long>((n + 255) / 256, 152LL * 16), 256, 0, c->stream>>>(n, x, dinv,
                                                                                                 c->d_xs);
  if ((e = launch_tile<0>(c, a, c->d_y32, nullptr)) != cudaSuccess) return e;
  k_amr_finish32<<<g1(c->nvc), 256, 0, c->stream>>>(c->nvc, a.h, c->d_ss, c->d_sc, c->d_sv,
                                                     c->d_y32, x, dinv, y);
  return cudaGetLastError();
}

cudaError_t launch_amr_matvec32_ff(amps_gpu_ctx* c, const OpIn& in, float* wh, float* wl) {
  cudaError_t e = cudaMemsetAsync(c->d_y32, 0, sizeof(float) * 3 * c->nvc, c->stream);
  if (e != cudaSuccess) return e;
  ApplyArgs a = apply_args(c);
  const long long n = 3 * c->nvc;
  if (!c->d_xs && (e = cudaMalloc(reinterpret_cast<void**>(&c->d_xs), sizeof(float) * 2 * n)) != cudaSuccess)
    return e;
  a.xf = c->d_xs;
  TimedLaunch t(c, "matvec32", in.xf_ready ? 2 : 3);
  if (!in.xf_ready && (e = launch_in_f32(c, in, c->d_xs)) != cudaSuccess) return e;
  if ((e = launch_tile<0>(c, a, c->d_y32, nullptr)) != cudaSuccess) return e;
  k_amr_finish_ff<<<g1(c->nvc), 256, 0, c->stream>>>(c->nvc, a.h, c->d_ss, c->d_sc, c->d_svh, c->d_svl,
                                                      c->d_y32, in, wh, wl);
  return cudaGetLastError();
}

cudaError_t launch_amr_rhs(amps_gpu_ctx* c) {
  cudaError_t e = cudaMemsetAsync(c->d_rhs, 0, sizeof(double) * 3 * c->nvc, c->stream);
  if (e != cudaSuccess) return e;
  ApplyArgs a = apply_args(c);
  a.x = c->d_En;
  a.dinv = nullptr;
  a.Bcen = c->d_Bc;
  TimedLaunch t(c, "rhs", 3);
  if ((e = split_input(c, c->d_En, nullptr, a)) != cudaSuccess) return e;
  if ((e = launch_tile<2>(c, a, nullptr, c->d_rhs)) != cudaSuccess) return e;
  k_amr_constraint<<<g1(c->nvc), 256, 0, c->stream>>>(c->nvc, a.h, nullptr, nullptr, c->d_rhs, 1);
  return cudaGetLastError();
}

cudaError_t launch_amr_jacobi(amps_gpu_ctx* c) {
  cudaError_t e = cudaMemsetAsync(c->d_dinv, 0, sizeof(double) * 3 * c->nvc, c->stream);
  if (e != cudaSuccess) return e;
  ApplyArgs a = apply_args(c);
  TimedLaunch t(c, "jacobi", 2);
  DiagK K{};
  for (int sc = 0; sc < kMaxScale; sc++) {
    const double dx = c->dxf * (double)(1 << sc), V = dx * dx * dx;
    K.base[sc] = (float)(V * (0.125 + a.th2dt2 / (8.0 * dx * dx)));
    K.fv[sc] = (float)(a.f * V);
  }
  k_amr_diag<<<g1(c->ncor), 256, 0, c->stream>>>(c->ncor, c->nvc, c->d_ctab, a.h, c->d_bscale,
                                                  c->d_cellM, K, c->d_dinv);
  k_amr_invert_diag<<<g1(c->nvc), 256, 0, c->stream>>>(c->nvc, a.h, c->d_dinv);
  return cudaGetLastError();
}

cudaError_t launch_amr_update_b(amps_gpu_ctx* c) {
  TimedLaunch t(c, "update_b");
  k_amr_update_b<<<g1(c->ncor), 256, 0, c->stream>>>(c->ncor, c->nvc, c->d_ctab, hang_of(c),
                                                      c->d_bdx, c->d_Eh, c->d_Bc, c->d_Bc2,
                                                      c->cfg.dt);
  if (c->mesh_open) {
    const int* nf = c->amrdev.nfine;
    for (int pass = 0; pass <= (c->neumann ? 3 : 0); pass++)
      k_amr_bnd_b<<<g1(c->ncor), 256, 0, c->stream>>>(c->ncor, c->d_borg, c->d_bscale, nf[0], nf[1], nf[2],
                                                       c->mesh_open, c->neumann, pass, c->d_Bc, c->d_Bc2);
  }
  return cudaGetLastError();
}

cudaError_t launch_amr_c2n(amps_gpu_ctx* c, const double* Bcen, double* Bcor) {
  // the GMRES work vector holds the weights (3*nvc >= nvc doubles)
  double* wsum = c->d_w;
  cudaError_t e = cudaMemsetAsync(Bcor, 0, sizeof(double) * 3 * c->nvc, c->stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(wsum, 0, sizeof(double) * c->nvc, c->stream);
  if (e != cudaSuccess) return e;
  TimedLaunch t(c, "c2n", 3);
  k_amr_c2n_acc<<<g1(c->ncor), 256, 0, c->stream>>>(c->ncor, c->nvc, c->d_ctab, c->d_bdx, Bcen,
                                                     Bcor, wsum);
  k_amr_c2n_div<<<g1(c->nvc), 256, 0, c->stream>>>(c->nvc, wsum, Bcor);
  k_amr_fix_hanging<<<g1(c->nvc), 256, 0, c->stream>>>(c->nvc, hang_of(c), Bcor);
  return cudaGetLastError();
}

cudaError_t launch_amr_update_e(amps_gpu_ctx* c) {
  cudaError_t e = cudaMemsetAsync(c->d_energy + 1, 0, sizeof(double), c->stream);
  if (e != cudaSuccess) return e;
  TimedLaunch t(c, "update_e", 3);
  k_amr_update_e<<<g1(c->nvc), 256, 0, c->stream>>>(c->nvc, c->d_Eh, c->d_En, c->cfg.theta);
  k_amr_fix_hanging<<<g1(c->nvc), 256, 0, c->stream>>>(c->nvc, hang_of(c), c->d_En);
  k_amr_wave_energy<<<g1(c->ncor), 256, 0, c->stream>>>(c->ncor, c->nvc, c->d_ctab, c->d_bdx,
                                                         c->d_En, c->d_Bc, c->d_energy + 1);
  return cudaGetLastError();
}

// E^{n+theta} = E^n + dE with hanging corners re-interpolated
cudaError_t launch_amr_fix_hanging(amps_gpu_ctx* c, double* F) {
  k_amr_fix_hanging<<<g1(c->nvc), 256, 0, c->stream>>>(c->nvc, hang_of(c), F);
  return cudaGetLastError();
}
