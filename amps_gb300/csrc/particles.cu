// Particle kernels of the ECSIM hot path on sm_103a.
//
// Particle layout: every cell owns a slot range [base[c], base[c+1]) of the
// FP32 SoA arrays; its cnt[c] particles sit at the front, the rest is slack
// (species byte 0xFF marks an empty slot).  Almost every particle stays in its
// cell during a step, so the step never re-sorts the whole population:
//
//   k_push_deposit<DEP,AMR,CB>
//                        one warp per cell: Lapenta2017 push of the cell's
//                        particles (src/pic/pic_mover_boris.cpp:876-1120) with
//                        E^{n+theta} and corner B^n gathered from a per-block
//                        stencil staged by one bulk (TMA) copy (CB: B^n from a
//                        staged stencil of the block's cell centres,
//                        CellCentered::Linear); particles that stay are
//                        compacted in place and, when DEP, deposited right away
//                        with ProcessCell's terms
//                        (pic_field_solver_ecsim.cpp:1882-2438); particles that
//                        leave are written into the slack of their destination
//                        cell (findTreeNode/FindCellIndex rules,
//                        meshAMRgeneric.h:2256-2320,2852-2883, periodic wrap of
//                        pic_bc_periodic.cpp:86-178), or to an overflow list
//   k_arrivals<DEP,CHUNK,CB>
//                        one CTA per block layer: the cells with arrivals are
//                        listed, warps take them from a shared counter, deposit
//                        the arrivals, move them behind the stayers, update cnt
//   k_ovf_place, k_relayout_cells
//                        slack overflow: overflowed arrivals into the slots
//                        their cells' movers vacated (deposited there); when a
//                        cell is full, every cell copied to new offsets in the
//                        other buffer
//   k_deposit<CB>        full ProcessCell pass over the compact layout
//                        (UpdateJMassMatrix without a preceding push)
//   k_assemble           per-cell partial sums -> 243-term corner mass matrix
//                        and corner J in FP64 (:2362-2426, shared corners summed)
//   rebuild              counting sort of an unsorted list into the slotted
//                        layout: import, and the positions the div E
//                        correction moves
//
// Deposition arithmetic: per particle the 27 distinct trilinear weight
// monomials, k*alpha (9), the 8 corner weights and q*alpha*v are staged in
// shared memory; 27 lanes each own a 3 x 3 tile of the 27x9 monomial block of
// the mass matrix and 3 lanes a 3 x 3 tile of the 8x3 current block, and
// accumulate it in registers over chunks of 32 particles (deposit_core.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "common.cuh"
#include "deposit_core.cuh"

namespace {



// SoA view of one particle buffer
struct PBuf {
  float* u[3];
  float* v[3];
  uint8_t* sp;
  float* wc;    // may be null
  uint32_t* id; // may be null
};

PBuf pbuf(amps_gpu_ctx* c, int which) {
  PBuf b;
  for (int q = 0; q < 3; q++) {
    b.u[q] = c->d_u[which][q];
    b.v[q] = c->d_v[which][q];
  }
  b.sp = c->d_sp[which];
  b.wc = c->has_wcorr ? c->d_wc[which] : nullptr;
  b.id = c->cfg.track_ids ? c->d_id[which] : nullptr;
  return b;
}

__device__ __forceinline__ void copy_particle(const PBuf& s, long long ps, const PBuf& d,
                                              long long pd) {
#pragma unroll
  for (int q = 0; q < 3; q++) {
    d.u[q][pd] = s.u[q][ps];
    d.v[q][pd] = s.v[q][ps];
  }
  d.sp[pd] = s.sp[ps];
  if (d.wc) d.wc[pd] = s.wc[ps];
  if (d.id) d.id[pd] = s.id[ps];
}

__device__ __forceinline__ float clamp_below8(float u) {
  return u < 8.0f ? u : 7.99999952316284180f;  // nextafterf(8, 0)
}

// AMR destination of a particle that left block b: unwrapped block-local
// offset un (cell units of b) -> position on the finest lattice (exact: the
// scale is a power of two), leaf block from the fine map, offset in that
// block's cell units (one rounding).  Periodic wrap moves the lattice position
// by whole domain lengths, which enter as integers.  Returns -1 when the
// particle left the domain through a face of an open axis (bit d of open).
__device__ __forceinline__ int amr_dest(const AmrDev& m, int b, float un[3], int ic[3], int open) {
  const float fs = (float)__ldg(m.bscale + b);
  int F[3], shift[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const int g = __ldg(m.borg + 3 * b + d) + (int)floorf(un[d] * fs);
    const int n = m.nfine[d];
    if (((open >> d) & 1) && (g < 0 || g >= n)) return -1;
    int w = g % n;
    if (w < 0) w += n;
    F[d] = w;
    shift[d] = g - w;
  }
  const int nb0 = m.nfine[0] >> 3, nb1 = m.nfine[1] >> 3;
  const int bn = __ldg(m.fine_map + (F[0] >> 3) + nb0 * ((F[1] >> 3) + nb1 * (F[2] >> 3)));
  const float inv = 1.0f / (float)__ldg(m.bscale + bn);  // exact: power of two
#pragma unroll
  for (int d = 0; d < 3; d++) {
    const int delta = __ldg(m.borg + 3 * bn + d) + shift[d] - __ldg(m.borg + 3 * b + d);
    const float u = clamp_below8(fmaxf((un[d] * fs - (float)delta) * inv, 0.0f));
    un[d] = u;
    ic[d] = min((int)u, AMPS_NC - 1);
  }
  return bn;
}

// Warp-aggregated reservation: one atomic per distinct key among active lanes;
// ranks inside the warp follow lane order.  Returns the reserved index.
__device__ __forceinline__ int warp_reserve(bool active, int key, int* __restrict__ counter) {
  const unsigned act = __ballot_sync(0xffffffffu, active);
  int r = -1;
  if (active) {
    const unsigned peers = __match_any_sync(act, key);
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if ((int)(threadIdx.x & 31) == leader) base = atomicAdd(counter + key, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    r = base + __popc(peers & lanemask_lt());
  }
  return r;
}

// ---------------------------------------------------------------------------
// Per block: the corner stencils (push: E^{n+theta}, corner B^n; deposit:
// corner B^{n+1}) and, with centre B (cp != nullptr), the centre stencils of
// B^n (Bcp) and B^{n+1} (Bcc) over the block's cells and the +-1 halo, centre
// (i, j, k) in -1..8 at (i+1) + 10 ((j+1) + 10 (k+1)).
__global__ void k_pack_stencils(int nb, long long ncor, const int* __restrict__ nbr,
                                const double* __restrict__ Eh, const double* __restrict__ Bprev,
                                const double* __restrict__ Bcur, float* __restrict__ sp,
                                float* __restrict__ sd, const double* __restrict__ Bcp,
                                const double* __restrict__ Bcc, float4* __restrict__ cp,
                                float4* __restrict__ cc) {
  const int b = blockIdx.x;
  if (cp) {
    for (int s = threadIdx.x; s < AMPS_CSC; s += blockDim.x) {
      const int cid = local_id(nbr, b, s % 10 - 1, (s / 10) % 10 - 1, s / 100 - 1);
      cp[(size_t)b * AMPS_CSC + s] =
          make_float4((float)Bcp[cid], (float)Bcp[ncor + cid], (float)Bcp[2 * ncor + cid], 0.f);
      cc[(size_t)b * AMPS_CSC + s] =
          make_float4((float)Bcc[cid], (float)Bcc[ncor + cid], (float)Bcc[2 * ncor + cid], 0.f);
    }
  }
  for (int s = threadIdx.x; s < AMPS_SC; s += blockDim.x) {
    const int i = s % 9, j = (s / 9) % 9, k = s / 81;
    const int cid = local_id(nbr, b, i, j, k);
    float4* op = reinterpret_cast<float4*>(sp + ((size_t)b * AMPS_SC + s) * AMPS_PUSH_STRIDE);
    op[0] = make_float4((float)Eh[cid], (float)Eh[ncor + cid], (float)Eh[2 * ncor + cid],
                        (float)Bprev[cid]);
    op[1] = make_float4((float)Bprev[ncor + cid], (float)Bprev[2 * ncor + cid], 0.f, 0.f);
    reinterpret_cast<float4*>(sd)[(size_t)b * AMPS_SC + s] =
        make_float4((float)Bcur[cid], (float)Bcur[ncor + cid], (float)Bcur[2 * ncor + cid], 0.f);
  }
}

// ---------------------------------------------------------------------------
struct StepArgs {
  const int* nbr;
  const int* base;
  int* cnt;
  int* arr;
  int* stay;
  const float* st_push;
  const float* st_dep;
  const float4* st_cprev;  // centre B stencils (centre-B runs), else nullptr
  const float4* st_ccur;
  PBuf p;         // current slots
  PBuf ovf;       // overflow list (the other buffer)
  int* ovf_key;
  float* cellM; float* cellJ;
  double* energy;
  unsigned long long* flags;  // [0] far, [1] near-face, [2] device error, [3] overflow count
  float dtdx[3];
  float inv_vol;
  long long ovf_cap;
  SpeciesTab st;
  AmrDev amr;     // fine_map == nullptr on uniform meshes
  int open;       // bit d: axis d is open (particles leaving the domain are deleted)
  int nbk[3];     // blocks per axis (uniform meshes)
};

// A uniform-mesh particle of block b whose destination lies o (in -1..1 per
// axis) blocks away leaves the domain through a face of an open axis.
__device__ __forceinline__ bool leaves_open_face(const StepArgs& a, int b, const int o[3]) {
  const int bc[3] = {b % a.nbk[0], (b / a.nbk[0]) % a.nbk[1], b / (a.nbk[0] * a.nbk[1])};
#pragma unroll
  for (int d = 0; d < 3; d++)
    if (((a.open >> d) & 1) && ((o[d] < 0 && bc[d] == 0) || (o[d] > 0 && bc[d] == a.nbk[d] - 1)))
      return true;
  return false;
}

// 1/dx^3 of block b
__device__ __forceinline__ float block_inv_vol(const StepArgs& a, int b) {
  return a.amr.binvvol ? __ldg(a.amr.binvvol + b) : a.inv_vol;
}

// Lapenta2017 velocity update v' = 2 alpha (v + h E) - v (Eqs. D.3, D.8)
__device__ __forceinline__ void lapenta(float h, const float E[3], const float B[3], float v[3]) {
  const float h2 = h * h;
  const float c0 = 1.0f / (1.0f + h2 * (B[0] * B[0] + B[1] * B[1] + B[2] * B[2]));
  const float P0 = -h * B[0], P1 = -h * B[1], P2 = -h * B[2];
  const float t0 = fmaf(h, E[0], v[0]), t1 = fmaf(h, E[1], v[1]), t2 = fmaf(h, E[2], v[2]);
  const float bt = h2 * (B[0] * t0 + B[1] * t1 + B[2] * t2);
  const float a0 = c0 * (t0 + B[0] * bt + (-P2 * t1 + P1 * t2));
  const float a1 = c0 * (t1 + B[1] * bt + (P2 * t0 - P0 * t2));
  const float a2 = c0 * (t2 + B[2] * bt + (-P1 * t0 + P0 * t1));
  v[0] = 2.f * a0 - v[0];
  v[1] = 2.f * a1 - v[1];
  v[2] = 2.f * a2 - v[2];
}

// CB: the particles see B interpolated from the cell centres (B^n from the
// centre stencil for the push, B^{n+1} for the deposit); E from the corners.
template <bool DEP, bool AMR, bool CB = false>
__global__ void __launch_bounds__(256, 2) k_push_deposit(StepArgs a) {
  extern __shared__ __align__(16) float4 s_dyn[];
  constexpr int kDepSC = CB ? AMPS_CSC : AMPS_SC;
  float4* s_push = s_dyn;                         // 729 x 2 float4
  float4* s_dep = s_dyn + 2 * AMPS_SC;            // 729 float4 corners, or 1000 centres (CB)
  float4* s_cprev = s_dep + kDepSC;               // 1000 float4 centres of B^n (CB)
  float* s_rec = reinterpret_cast<float*>(s_cprev + (CB ? AMPS_CSC : 0));  // kWarps x kFields x kFS
  __shared__ __align__(8) uint64_t bar;
  __shared__ double s_en[kWarps];
  const int b = blockIdx.x, k = blockIdx.y;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const uint32_t bp = AMPS_SC * AMPS_PUSH_STRIDE * sizeof(float);
  const uint32_t bd = DEP ? kDepSC * 4 * sizeof(float) : 0;
  const uint32_t bc = CB ? AMPS_CSC * sizeof(float4) : 0;
  const int j = wid;
  // slot range and occupancy of the row's 8 cells, one lane per cell
  int mb0 = 0, mn0 = 0;
  if (lane < AMPS_NC) {
    const long long cl = (long long)b * AMPS_CPB + lane + AMPS_NC * (j + AMPS_NC * k);
    mb0 = a.base[cl];
    mn0 = a.cnt[cl];
  }
  // software pipeline over the row's chunks: the next chunk's particles (the
  // next 32 of this cell, or the first 32 of the next cell) are loaded while
  // this one is processed; its slots lie above every slot this chunk writes
  float pu[3] = {0.f, 0.f, 0.f}, pv[3] = {0.f, 0.f, 0.f};
  int ps = 0;
  float pwc = 1.0f;
  uint32_t pid = 0;
  int pf_cell = 0;  // cell whose chunk the prefetch registers hold
  auto prefetch = [&](int c, int q) {
    const int cb = __shfl_sync(0xffffffffu, mb0, c), cn = __shfl_sync(0xffffffffu, mn0, c);
    pf_cell = c;
    if (q < cn) {
      const int pn = cb + q;
#pragma unroll
      for (int d = 0; d < 3; d++) { pu[d] = a.p.u[d][pn]; pv[d] = a.p.v[d][pn]; }
      ps = a.p.sp[pn];
      pwc = a.p.wc ? a.p.wc[pn] : 1.0f;
      pid = a.p.id ? a.p.id[pn] : 0u;
    }
  };
  prefetch(0, lane);  // in flight while the stencils are staged
  const void* dep_src = CB ? (const void*)(a.st_ccur + (size_t)b * AMPS_CSC)
                           : (const void*)(a.st_dep + (size_t)b * AMPS_SC * AMPS_DEP_STRIDE);
  if (!stage_stencils(&bar, s_push, a.st_push + (size_t)b * AMPS_SC * AMPS_PUSH_STRIDE, bp, s_dep,
                      dep_src, bd, a.flags, s_cprev, CB ? a.st_cprev + (size_t)b * AMPS_CSC : nullptr,
                      bc))
    return;
  float* rec = s_rec + wid * kFields * kFS;
  int fA, fB;
  lane_fields(lane, fA, fB);
  FF en_row{0.f, 0.f};  // float pair across the row's cells, FP64 in the CTA reduction
  unsigned long long n_far = 0, n_near = 0, n_del = 0;
  const float inv_vol = block_inv_vol(a, b);
  const float bdtdx = AMR ? __ldg(a.amr.bdtdx + b) : 0.0f;
  for (int i = 0; i < AMPS_NC; i++) {
    const long long cid = (long long)b * AMPS_CPB + i + AMPS_NC * (j + AMPS_NC * k);
    const int b0 = __shfl_sync(0xffffffffu, mb0, i), n0 = __shfl_sync(0xffffffffu, mn0, i);
    Tile tile;
    tile.zero();
    int nst = 0;
    if (pf_cell != i) prefetch(i, lane);  // the previous cell was empty
    for (int q0 = 0; q0 < n0; q0 += 32) {
      const int p = b0 + q0 + lane;
      const bool act = q0 + lane < n0;
      float u[3] = {pu[0], pu[1], pu[2]}, v[3] = {pv[0], pv[1], pv[2]};
      int s = ps, key = -1;
      float wcv = pwc;
      uint32_t idv = pid;
      if (q0 + 32 < n0)
        prefetch(i, q0 + 32 + lane);
      else if (i + 1 < AMPS_NC)
        prefetch(i + 1, lane);
      if (act) {
        // gather E^{n+theta}, B^n at the old position
        int ic[3];
        float f[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
          ic[d] = min(max((int)u[d], 0), AMPS_NC - 1);
          f[d] = u[d] - (float)ic[d];
        }
        // E and B as three packed pairs (E0 E1) (E2 B0) (B1 B2), the layout of a
        // stencil corner's two float4s, accumulated by packed FMAs
        unsigned long long eb[2][3] = {{0ull, 0ull, 0ull}, {0ull, 0ull, 0ull}};  // z = 0, 1 layers
#pragma unroll
        for (int cc = 0; cc < 2; cc++)
#pragma unroll
          for (int bb = 0; bb < 2; bb++)
#pragma unroll
            for (int aa = 0; aa < 2; aa++) {
              const float w = (aa ? f[0] : 1.f - f[0]) * (bb ? f[1] : 1.f - f[1]) *
                              (cc ? f[2] : 1.f - f[2]);
              const int sidx = (ic[0] + aa) + 9 * (ic[1] + bb) + 81 * (ic[2] + cc);
              const ulonglong2 q0v = reinterpret_cast<const ulonglong2*>(s_push)[2 * sidx];
              unsigned long long ww;
              asm("mov.b64 %0, {%1, %1};" : "=l"(ww) : "f"(w));
              ffma2(eb[cc][0], ww, q0v.x);
              ffma2(eb[cc][1], ww, q0v.y);
              if (!CB) {
                const ulonglong2 q1v = reinterpret_cast<const ulonglong2*>(s_push)[2 * sidx + 1];
                ffma2(eb[cc][2], ww, q1v.x);
              }
            }
        float eb_f[6];
#pragma unroll
        for (int t = 0; t < 3; t++) {
          const float2 lo = *reinterpret_cast<const float2*>(&eb[0][t]);
          const float2 hi = *reinterpret_cast<const float2*>(&eb[1][t]);
          eb_f[2 * t] = lo.x + hi.x;
          eb_f[2 * t + 1] = lo.y + hi.y;
        }
        const float E[3] = {eb_f[0], eb_f[1], eb_f[2]};
        float B[3] = {eb_f[3], eb_f[4], eb_f[5]};
        if (CB) centre_b(s_cprev, u[0], u[1], u[2], B);
        lapenta(a.st.qdt2m[s], E, B, v);
        bool far = false, nearf = false;
        int nbk = b;
        if (AMR) {
          bool out = false;
#pragma unroll
          for (int d = 0; d < 3; d++) {
            u[d] = fmaf(v[d], bdtdx, u[d]);
            const int od = (int)floorf(u[d] * 0.125f);
            if (od > 1 || od < -1) far = true;
            if (!(u[d] >= 0.0f && u[d] < 8.0f)) out = true;
            ic[d] = min((int)u[d], AMPS_NC - 1);
          }
          if (out) nbk = amr_dest(a.amr, b, u, ic, a.open);
#pragma unroll
          for (int d = 0; d < 3; d++)
            if (fabsf(u[d] - rintf(u[d])) < 4.76837158203125e-7f) nearf = true;
        } else {
          int o[3];
#pragma unroll
          for (int d = 0; d < 3; d++) {
            float un = fmaf(v[d], a.dtdx[d], u[d]);
            int od = (int)floorf(un * 0.125f);
            if (od > 1 || od < -1) far = true;
            od = max(-1, min(1, od));
            un -= 8.0f * (float)od;
            un = clamp_below8(fmaxf(un, 0.0f));
            o[d] = od;
            u[d] = un;
            ic[d] = min((int)un, AMPS_NC - 1);
            if (fabsf(un - rintf(un)) < 4.76837158203125e-7f) nearf = true;
          }
          if (o[0] | o[1] | o[2])
            nbk = (a.open && leaves_open_face(a, b, o)) ? -1
                                                        : __ldg(a.nbr + b * 27 + nbr_slot(o[0], o[1], o[2]));
        }
        if (far) n_far++;
        if (nearf) n_near++;
        // nbk < 0: the particle left the domain through an open face and is
        // deleted (no slot, no deposit)
        if (nbk >= 0) key = nbk * AMPS_CPB + ic[0] + AMPS_NC * (ic[1] + AMPS_NC * ic[2]);
        else n_del++;
      }
      const bool stays = act && key == (int)cid;
      const unsigned smask = __ballot_sync(0xffffffffu, stays);
      const int spos = __popc(smask & lanemask_lt());
      __syncwarp();
      if (stays) {
        const long long d = b0 + nst + spos;
#pragma unroll
        for (int dd = 0; dd < 3; dd++) { a.p.u[dd][d] = u[dd]; a.p.v[dd][d] = v[dd]; }
        if (d != p) {
          a.p.sp[d] = (uint8_t)s;
          if (a.p.wc) a.p.wc[d] = wcv;
          if (a.p.id) a.p.id[d] = idv;
        }
      }
      // every lane stages its position; only stayers carry weight (movers are
      // deposited by k_arrivals in their destination cell)
      if (DEP)
        stage_fields<kFS, CB>(rec, lane, s_dep, u[0], u[1], u[2], v[0], v[1], v[2], act ? s : 0,
                          stays ? wcv : 0.f, i, j, k, a.st, inv_vol, en_row);
      // movers: slack of the destination cell, else the overflow list
      const bool mover = act && !stays && key >= 0;
      // one reservation per mover (a chunk has a few): no warp-wide key match
      const int slot = mover ? atomicAdd(a.arr + key, 1) : 0;
      if (mover) {
        const int cb = a.base[key], ccap = a.base[key + 1] - cb, cn = a.cnt[key];
        if (slot < ccap - cn) {
          const long long d = (long long)cb + ccap - 1 - slot;
#pragma unroll
          for (int dd = 0; dd < 3; dd++) { a.p.u[dd][d] = u[dd]; a.p.v[dd][d] = v[dd]; }
          a.p.sp[d] = (uint8_t)s;
          if (a.p.wc) a.p.wc[d] = wcv;
          if (a.p.id) a.p.id[d] = idv;
        } else {
          const unsigned long long o = atomicAdd(a.flags + 3, 1ull);
          if ((long long)o < a.ovf_cap) {
#pragma unroll
            for (int dd = 0; dd < 3; dd++) { a.ovf.u[dd][o] = u[dd]; a.ovf.v[dd][o] = v[dd]; }
            a.ovf.sp[o] = (uint8_t)s;
            if (a.ovf.wc) a.ovf.wc[o] = wcv;
            if (a.ovf.id) a.ovf.id[o] = idv;
            a.ovf_key[o] = key;
          } else {
            atomicAdd(a.flags + 2, 1ull);
          }
        }
      }
      const int cst = __popc(smask);
      if (DEP) {
        __syncwarp();
        if (cst > 0) tile.accumulate<kFS>(rec, (min(32, n0 - q0) + 3) & ~3, fA, fB);
        __syncwarp();
      }
      nst += cst;
    }
    // vacated slots become holes
    for (int t = nst + lane; t < n0; t += 32) a.p.sp[b0 + t] = kHole;
    if (lane == 0) a.stay[cid] = nst;
    if (DEP) tile.flush(lane, a.cellM, a.cellJ, cid);
  }
  if (n_far) atomicAdd(a.flags + 0, n_far);
  if (n_near) atomicAdd(a.flags + 1, n_near);
  if (n_del) atomicAdd(a.flags + 5, n_del);
  if (DEP) reduce_energy(ff_value(en_row), s_en, a.energy);
}

// ---------------------------------------------------------------------------
// Injection through open faces: the OpenFlow boundary of the reference
// (PIC::BC::ExternalBoundary::OpenFlow, src/pic/pic_bc.cpp:330-420) on every
// boundary cell face of an injection source: a Poisson process in time at the
// rate CalculateInjectionRate_MaxwellianDistribution (pic_bc.cpp:215) x face
// area / macro-particle weight; each particle at a uniform point of the face
// with the velocity of InjectMaxwellianDistribution
// (src/pic/pic_vel_distribution.cpp:49-161), then moved by the Lapenta2017
// mover for the rest of the step, and placed in its destination cell like a
// mover (k_arrivals deposits it).  Random numbers: a counter-based stream per
// (seed, step, source, face cell), inj_uniform below; the FP64 oracle restates
// the same stream.  One thread per (source, boundary cell face).
constexpr int kMaxInj = 8;
struct InjDev {
  int face, spec, ncell, first;  // first: index of the source's first thread
  double rate;                   // particles per unit face area per unit time (/weight)
  double drift[3], beta;         // bulk velocity; beta = 1 / (sqrt(2) vth)
};
struct InjArgs {
  InjDev src[kMaxInj];
  int nsrc, nthreads;
  double dt, dx[3];
  int nbk[3];
  unsigned long long seed;
  const unsigned long long* step;  // [0] step counter, [1] next particle id
};

__device__ __forceinline__ unsigned long long inj_mix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
// uniform in (0, 1) from draw d of the stream key
__device__ __forceinline__ double inj_uniform(unsigned long long key, unsigned& d) {
  return ((double)(inj_mix(key + (d++)) >> 11) + 0.5) * 0x1.0p-53;
}

__global__ void __launch_bounds__(128) k_inject(StepArgs a, InjArgs g) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nthreads) return;
  int s = 0;
  while (s + 1 < g.nsrc && t >= g.src[s + 1].first) s++;
  const InjDev S = g.src[s];
  const int c = t - S.first;
  const int ax = S.face >> 1, hi = S.face & 1, ta = (ax + 1) % 3, tb = (ax + 2) % 3;
  const bool amr = a.amr.fine_map != nullptr;
  // face cells (uniform) or finest-lattice face patches (AMR), each its own stream
  const int NT = amr ? a.amr.nfine[ta] : 8 * g.nbk[ta];
  const int it = c % NT, ib = c / NT;  // tangential cell coordinates
  const double area = g.dx[ta] * g.dx[tb];
  const double R = S.rate * area;
  if (!(R > 0.0)) return;
  double nrm[3] = {0.0, 0.0, 0.0};
  nrm[ax] = hi ? 1.0 : -1.0;  // outward normal
  const unsigned long long key =
      inj_mix(inj_mix(inj_mix(g.seed) ^ *g.step) ^ (((unsigned long long)s << 40) | (unsigned long long)c));
  unsigned d = 0;
  double tt = 0.0;
  for (int k = 0; k < 4096; k++) {
    tt += -log(inj_uniform(key, d)) / R;
    if (tt >= g.dt) break;
    const double c0 = inj_uniform(key, d), c1 = inj_uniform(key, d);
    // velocity: InjectMaxwellianDistribution (3D branch)
    double v[3] = {0.0, 0.0, 0.0};
    bool ok = false;
    for (int outer = 0; outer < 64 && !ok; outer++) {
      const double dot = S.drift[0] * nrm[0] + S.drift[1] * nrm[1] + S.drift[2] * nrm[2];
      const double sc = S.beta * fabs(dot);
      double u = 0.0, acc = 0.0;
      bool got = false;
      for (int tries = 0; tries < 4096 && !got; tries++) {
        if (dot <= 0.0) {
          int q = 0;
          do u = -10.0 + 20.0 * inj_uniform(key, d); while (u + sc <= 0.0 && ++q < 4096);
          const double cc = sqrt(2.0 + sc * sc);
          acc = 2.0 * (u + sc) / (sc + cc) * exp(0.5 + 0.5 * sc * (sc - cc) - u * u);
        } else {
          int q = 0;
          do u = -10.0 + 20.0 * inj_uniform(key, d); while (u + sc >= 0.0 && ++q < 4096);
          const double cc = 0.5 * (-sqrt(sc * sc + 2.0) - sc);
          acc = (u + sc) * exp(-u * u) / (cc + sc) / exp(-cc * cc);
        }
        got = !(acc < inj_uniform(key, d));
      }
      if (!got) break;
      double v1[3], v2[3], v3[3];
      for (int q = 0; q < 3; q++) v3[q] = -(fabs(u + sc) / S.beta) * nrm[q];
      if (fabs(nrm[0]) > 1.0e-3) {
        v2[0] = nrm[1]; v2[1] = -nrm[0]; v2[2] = 0.0;
      } else {
        v2[0] = 0.0; v2[1] = nrm[2]; v2[2] = -nrm[1];
      }
      double l2 = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
      for (int q = 0; q < 3; q++) v2[q] /= l2;
      v1[0] = v2[1] * nrm[2] - v2[2] * nrm[1];
      v1[1] = -(v2[0] * nrm[2] - v2[2] * nrm[0]);
      v1[2] = v2[0] * nrm[1] - v2[1] * nrm[0];
      double l1 = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
      for (int q = 0; q < 3; q++) v1[q] /= l1;
      const double cm = sqrt(-log(inj_uniform(key, d))) / S.beta, cp = inj_uniform(key, d);
      const double d1 = S.drift[0] * v1[0] + S.drift[1] * v1[1] + S.drift[2] * v1[2];
      const double d2 = S.drift[0] * v2[0] + S.drift[1] * v2[1] + S.drift[2] * v2[2];
      const double kPi2 = 6.283185307179586476925286766559;
      for (int q = 0; q < 3; q++)
        v[q] = (cm * sin(kPi2 * cp) + d1) * v1[q] + (cm * cos(kPi2 * cp) + d2) * v2[q] + v3[q];
      ok = v[0] * nrm[0] + v[1] * nrm[1] + v[2] * nrm[2] < 0.0;
    }
    if (!ok) {
      atomicAdd(a.flags + 2, 1ull);  // sampling did not finish within its bounds
      return;
    }
    // position on the face, in the block-local cell units of the boundary cell's block
    int b;
    float u[3];
    u[ax] = hi ? 8.0f : 0.0f;
    const double pt = (it + c0), pb = (ib + c1);
    if (amr) {
      // the leaf block owning the patch's boundary cell (finest lattice)
      int F[3];
      F[ax] = hi ? a.amr.nfine[ax] - 1 : 0;
      F[ta] = it;
      F[tb] = ib;
      b = __ldg(a.amr.fine_map + (F[0] >> 3) + (a.amr.nfine[0] >> 3) * ((F[1] >> 3) + (a.amr.nfine[1] >> 3) * (F[2] >> 3)));
      const double sc = (double)__ldg(a.amr.bscale + b);
      u[ta] = (float)((pt - (double)__ldg(a.amr.borg + 3 * b + ta)) / sc);
      u[tb] = (float)((pb - (double)__ldg(a.amr.borg + 3 * b + tb)) / sc);
    } else {
      int bc[3];
      bc[ax] = hi ? g.nbk[ax] - 1 : 0;
      bc[ta] = (int)(pt / 8.0);
      u[ta] = (float)(pt - 8.0 * bc[ta]);
      bc[tb] = (int)(pb / 8.0);
      u[tb] = (float)(pb - 8.0 * bc[tb]);
      b = bc[0] + g.nbk[0] * (bc[1] + g.nbk[1] * bc[2]);
    }
    // Lapenta2017 for the rest of the step, fields from the block's packed stencil
    const float frac = (float)((g.dt - tt) / g.dt);
    float vf[3] = {(float)v[0], (float)v[1], (float)v[2]};
    {
      int ic[3];
      float f[3];
      for (int q = 0; q < 3; q++) {
        ic[q] = min(max((int)u[q], 0), AMPS_NC - 1);
        f[q] = u[q] - (float)ic[q];
      }
      float E[3] = {0.f, 0.f, 0.f}, B[3] = {0.f, 0.f, 0.f};
      for (int cc = 0; cc < 8; cc++) {
        const int ox = cc & 1, oy = (cc >> 1) & 1, oz = cc >> 2;
        const float w = (ox ? f[0] : 1.f - f[0]) * (oy ? f[1] : 1.f - f[1]) * (oz ? f[2] : 1.f - f[2]);
        const float* st = a.st_push + ((size_t)b * AMPS_SC + (ic[0] + ox) + 9 * ((ic[1] + oy) + 9 * (ic[2] + oz))) *
                                          AMPS_PUSH_STRIDE;
        E[0] = fmaf(w, st[0], E[0]);
        E[1] = fmaf(w, st[1], E[1]);
        E[2] = fmaf(w, st[2], E[2]);
        B[0] = fmaf(w, st[3], B[0]);
        B[1] = fmaf(w, st[4], B[1]);
        B[2] = fmaf(w, st[5], B[2]);
      }
      lapenta(a.st.qdt2m[S.spec] * frac, E, B, vf);
    }
    // move and locate (periodic wrap, deletion through open faces)
    int o[3], ic[3];
    bool far = false;
    int nbk = b;
    if (amr) {
      const float dtdx = __ldg(a.amr.bdtdx + b) * frac;
      for (int q = 0; q < 3; q++) u[q] = fmaf(vf[q], dtdx, u[q]);
      nbk = amr_dest(a.amr, b, u, ic, a.open);
      if (nbk < 0) continue;  // left the domain again at once
    } else {
    for (int q = 0; q < 3; q++) {
      float un = fmaf(vf[q], a.dtdx[q] * frac, u[q]);
      int od = (int)floorf(un * 0.125f);
      if (od > 1 || od < -1) far = true;
      od = max(-1, min(1, od));
      un -= 8.0f * (float)od;
      un = clamp_below8(fmaxf(un, 0.0f));
      o[q] = od;
      u[q] = un;
      ic[q] = min((int)un, AMPS_NC - 1);
    }
    if (far) atomicAdd(a.flags + 0, 1ull);
    if (o[0] | o[1] | o[2]) {
      if (a.open && leaves_open_face(a, b, o)) continue;  // left again at once
      nbk = __ldg(a.nbr + b * 27 + nbr_slot(o[0], o[1], o[2]));
    }
    }
    const int key2 = nbk * AMPS_CPB + ic[0] + AMPS_NC * (ic[1] + AMPS_NC * ic[2]);
    const uint32_t idv = (uint32_t)g.step[1] + (uint32_t)atomicAdd(a.flags + 6, 1ull);
    const int slot = atomicAdd(a.arr + key2, 1);
    const int cb = a.base[key2], ccap = a.base[key2 + 1] - cb, cn = a.cnt[key2];
    if (slot < ccap - cn) {
      const long long dd = (long long)cb + ccap - 1 - slot;
      for (int q = 0; q < 3; q++) { a.p.u[q][dd] = u[q]; a.p.v[q][dd] = vf[q]; }
      a.p.sp[dd] = (uint8_t)S.spec;
      if (a.p.wc) a.p.wc[dd] = 1.0f;
      if (a.p.id) a.p.id[dd] = idv;
    } else {
      const unsigned long long ov = atomicAdd(a.flags + 3, 1ull);
      if ((long long)ov < a.ovf_cap) {
        for (int q = 0; q < 3; q++) { a.ovf.u[q][ov] = u[q]; a.ovf.v[q][ov] = vf[q]; }
        a.ovf.sp[ov] = (uint8_t)S.spec;
        if (a.ovf.wc) a.ovf.wc[ov] = 1.0f;
        if (a.ovf.id) a.ovf.id[ov] = idv;
        a.ovf_key[ov] = key2;
      } else {
        atomicAdd(a.flags + 2, 1ull);
      }
    }
  }
}

__global__ void k_set_next_id(unsigned long long* step, unsigned long long n) {
  if (threadIdx.x == 0 && blockIdx.x == 0) step[1] = n;
}

// after the injection: next step, ids past the injected ones
__global__ void k_step_bump(unsigned long long* step, const unsigned long long* flags) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    step[0] += 1ull;
    step[1] += flags[6];
  }
}

// Arrivals: deposit (DEP), move behind the stayers, update the occupancy.
// A CTA takes the 64 cells of one block layer: one thread per cell loads its
// slot range and counts and updates the occupancy, the cells with arrivals are
// listed in shared memory, and the warps take listed cells one at a time from
// a shared counter, so a few busy cells do not hold idle warps at the CTA's
// final barrier.  Arrivals are few per cell (a few % of its particles), so
// records are staged in chunks of CHUNK lanes: at 16, a smaller record buffer
// and a 64-register cap (56 bytes of spills) let 4 CTAs share an SM, which
// hides more of the per-cell load latency (0.29 against 0.32 ms per launch
// with 3 CTAs on the 67.1M-particle AMR plasma); 32 (2 CTAs per SM) halves the
// chunks of cells with many arrivals.  The autotuner picks one on the run's
// own steps.
constexpr int kArrChunk = 16;
constexpr int kFSArr = kArrChunk + 4;  // field stride of staged fields at 16 lanes
constexpr int kLayer = AMPS_NC * AMPS_NC;

template <bool DEP, int CHUNK, bool CB = false>
__global__ void __launch_bounds__(256, CHUNK == 16 ? 4 : 2) k_arrivals(StepArgs a) {
  constexpr int FS = CHUNK + 4;  // field stride of the staged fields
  extern __shared__ __align__(16) float4 s_dyn[];
  float* s_rec = reinterpret_cast<float*>(s_dyn);
  __shared__ double s_en[kWarps];
  __shared__ int4 s_cell[kLayer];  // listed cell: layer index, first arrival slot, destination, count
  __shared__ int s_nw[2], s_next;
  const int b = blockIdx.x, k = blockIdx.y;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // the few arrivals read the block's B stencil from global memory (L2-resident:
  // 11.7 KB per block, 16 KB of centres) instead of waiting for a staged copy
  // at CTA start
  const float4* s_dep = CB ? a.st_ccur + (size_t)b * AMPS_CSC
                           : reinterpret_cast<const float4*>(a.st_dep) + (size_t)b * AMPS_SC;
  int4 cv = make_int4(0, 0, 0, 0);
  bool has = false;
  if (threadIdx.x < kLayer) {
    const long long cl = (long long)b * AMPS_CPB + threadIdx.x + kLayer * k;
    const int b0 = a.base[cl], cap = a.base[cl + 1] - b0, n0 = a.cnt[cl], nst = a.stay[cl];
    const int na = min(a.arr[cl], cap - n0);
    a.cnt[cl] = nst + max(0, na);
    a.arr[cl] = 0;
    has = na > 0;
    cv = make_int4(threadIdx.x, b0 + cap - na, b0 + nst, na);
  }
  const unsigned hm = __ballot_sync(0xffffffffu, has);
  if (lane == 0 && wid < 2) s_nw[wid] = __popc(hm);
  if (threadIdx.x == 0) s_next = 0;
  __syncthreads();
  if (has) s_cell[(wid ? s_nw[0] : 0) + __popc(hm & lanemask_lt())] = cv;
  const int ncell = s_nw[0] + s_nw[1];
  __syncthreads();
  float* rec = s_rec + wid * kFields * FS;
  int fA, fB;
  lane_fields(lane, fA, fB);
  FF en_w{0.f, 0.f};  // the warp's arrivals, as a float pair before the FP64 reduction
  const float inv_vol = block_inv_vol(a, b);
  for (;;) {
    int e = 0;
    if (lane == 0) e = atomicAdd(&s_next, 1);
    e = __shfl_sync(0xffffffffu, e, 0);
    if (e >= ncell) break;
    const int4 c = s_cell[e];
    const int i = c.x & (AMPS_NC - 1), j = c.x / AMPS_NC;
    const int src0 = c.y, dst0 = c.z, na = c.w;
    const long long cid = (long long)b * AMPS_CPB + c.x + kLayer * k;
    Tile tile;
    tile.zero();
    for (int q0 = 0; q0 < na; q0 += CHUNK) {
      const bool act = lane < CHUNK && q0 + lane < na;
      const long long ps = src0 + q0 + lane, pd = dst0 + q0 + lane;
      float u[3] = {0.f, 0.f, 0.f}, v[3] = {0.f, 0.f, 0.f};
      int s = 0;
      float wcv = 1.0f;
      uint32_t idv = 0;
      if (act) {
#pragma unroll
        for (int d = 0; d < 3; d++) { u[d] = a.p.u[d][ps]; v[d] = a.p.v[d][ps]; }
        s = a.p.sp[ps];
        if (a.p.wc) wcv = a.p.wc[ps];
        if (a.p.id) idv = a.p.id[ps];
      }
      __syncwarp();
      if (act) {
#pragma unroll
        for (int d = 0; d < 3; d++) { a.p.u[d][pd] = u[d]; a.p.v[d][pd] = v[d]; }
        a.p.sp[pd] = (uint8_t)s;
        if (a.p.wc) a.p.wc[pd] = wcv;
        if (a.p.id) a.p.id[pd] = idv;
      }
      if (DEP) {
        // positions past the chunk's arrivals stage zero weight
        if (lane < CHUNK)
          stage_fields<FS, CB>(rec, lane, s_dep, u[0], u[1], u[2], v[0], v[1], v[2], s,
                               act ? wcv : 0.f, i, j, k, a.st, inv_vol, en_w);
        __syncwarp();
        tile.accumulate<FS>(rec, (min(CHUNK, na - q0) + 3) & ~3, fA, fB);
        __syncwarp();
      }
    }
    // slots that held arrivals and are now beyond the new occupancy
    for (int t = lane; t < na; t += 32) {
      const int slot = src0 + t;
      if (slot >= dst0 + na) a.p.sp[slot] = kHole;
    }
    if (DEP) tile.flush_red(lane, rec, a.cellM, a.cellJ, cid);
  }
  if (DEP) reduce_energy(ff_value(en_w), s_en, a.energy);
}

// Overflow entries into the slots their cell's movers vacated.  The push and
// the arrivals give arrivals only a cell's slack (the slots past its occupancy
// at the start of the step), so a cell can overflow while the particles that
// left it freed slots; after the arrivals a cell's first cnt slots hold its
// particles and the rest of its range is free.  One warp per entry: a free
// slot is reserved on cnt, the particle written there and the entry's key set
// to -1.  Entries whose cell is full are counted in *left and stay in the list
// for the relayout, which files them in the same cell.  Every entry is
// deposited here like an arrival (DEP).
template <bool DEP, bool CB = false>
__global__ void __launch_bounds__(256) k_ovf_place(StepArgs a, long long n_ovf,
                                                   unsigned long long* left) {
  extern __shared__ __align__(16) float4 s_dyn[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const long long e = (long long)blockIdx.x * kWarps + wid;
  if (e >= n_ovf) return;  // the whole warp: no block-wide barrier follows
  const int key = a.ovf_key[e];
  const int b0 = a.base[key], cap = a.base[key + 1] - b0;
  int slot = 0;
  if (lane == 0) {
    slot = atomicAdd(a.cnt + key, 1);
    if (slot >= cap) atomicSub(a.cnt + key, 1);  // cnt never falls below cap again
  }
  slot = __shfl_sync(0xffffffffu, slot, 0);
  const bool fits = slot < cap;
  if (!fits && lane == 0) atomicAdd(left, 1ull);
  float u[3], v[3];
#pragma unroll
  for (int d = 0; d < 3; d++) { u[d] = a.ovf.u[d][e]; v[d] = a.ovf.v[d][e]; }
  const int s = a.ovf.sp[e];
  const float wcv = a.ovf.wc ? a.ovf.wc[e] : 1.0f;
  if (fits && lane == 0) {
    const long long d = (long long)b0 + slot;
#pragma unroll
    for (int q = 0; q < 3; q++) { a.p.u[q][d] = u[q]; a.p.v[q][d] = v[q]; }
    a.p.sp[d] = (uint8_t)s;
    if (a.p.wc) a.p.wc[d] = wcv;
    if (a.p.id) a.p.id[d] = a.ovf.id[e];
    a.ovf_key[e] = -1;
  }
  if (DEP) {
    float* rec = reinterpret_cast<float*>(s_dyn) + wid * kFields * kFSArr;
    int fA, fB;
    lane_fields(lane, fA, fB);
    const int b = key / AMPS_CPB, l = key % AMPS_CPB;
    const float4* s_dep = CB ? a.st_ccur + (size_t)b * AMPS_CSC
                             : reinterpret_cast<const float4*>(a.st_dep) + (size_t)b * AMPS_SC;
    FF en{0.f, 0.f};
    // the particle at position 0, zero weight at positions 1..3
    if (lane < 4)
      stage_fields<kFSArr, CB>(rec, lane, s_dep, u[0], u[1], u[2], v[0], v[1], v[2], s,
                           lane == 0 ? wcv : 0.f, l & (AMPS_NC - 1), (l / AMPS_NC) & (AMPS_NC - 1),
                           l / (AMPS_NC * AMPS_NC), a.st, block_inv_vol(a, b), en);
    __syncwarp();
    Tile tile;
    tile.zero();
    tile.accumulate<kFSArr>(rec, 4, fA, fB);
    __syncwarp();
    tile.flush_red(lane, rec, a.cellM, a.cellJ, key);
    if (lane == 0) atomicAdd(a.energy, ff_value(en));
  }
}

// Relayout kernels (particles_relayout): the unplaced overflow entries (key
// >= 0) counted per cell; one warp per cell copying its particles to the new
// offsets (pad + newb[c]); the unplaced entries behind them.
__global__ void __launch_bounds__(256) k_ovf_count(long long n_ovf, const int* __restrict__ key,
                                                   int* __restrict__ count) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e < n_ovf && key[e] >= 0) atomicAdd(count + key[e], 1);
}

// Each lane loads its kRelayoutRound particles of a round before it stores any
// (the source and destination buffers are distinct): the copy is bound by the
// loads in flight, and one particle per lane at a time ran at a third of the
// rate (1.5 against 4.3 TB/s on 584M particles).
constexpr int kRelayoutRound = 4;
__global__ void __launch_bounds__(256) k_relayout_cells(long long ncell, const int* __restrict__ base,
                                                        const int* __restrict__ cnt,
                                                        const int* __restrict__ newb, long long pad,
                                                        PBuf s, PBuf d) {
  const long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= ncell) return;
  const long long ob = base[c], nb = pad + newb[c];
  const int n = cnt[c];
  for (int q0 = 0; q0 < n; q0 += 32 * kRelayoutRound) {
    float u[kRelayoutRound][3], v[kRelayoutRound][3], w[kRelayoutRound];
    uint32_t id[kRelayoutRound];
    uint8_t sp[kRelayoutRound];
#pragma unroll
    for (int r = 0; r < kRelayoutRound; r++) {
      const long long q = q0 + 32 * r + lane;
      if (q < n) {
#pragma unroll
        for (int k = 0; k < 3; k++) { u[r][k] = __ldg(s.u[k] + ob + q); v[r][k] = __ldg(s.v[k] + ob + q); }
        sp[r] = __ldg(s.sp + ob + q);
        w[r] = s.wc ? __ldg(s.wc + ob + q) : 0.f;
        id[r] = s.id ? __ldg(s.id + ob + q) : 0u;
      }
    }
#pragma unroll
    for (int r = 0; r < kRelayoutRound; r++) {
      const long long q = q0 + 32 * r + lane;
      if (q < n) {
#pragma unroll
        for (int k = 0; k < 3; k++) { d.u[k][nb + q] = u[r][k]; d.v[k][nb + q] = v[r][k]; }
        d.sp[nb + q] = sp[r];
        if (d.wc) d.wc[nb + q] = w[r];
        if (d.id) d.id[nb + q] = id[r];
      }
    }
  }
}

__global__ void __launch_bounds__(256) k_ovf_file(long long n_ovf, const int* __restrict__ key,
                                                  const int* __restrict__ newb, long long pad,
                                                  int* __restrict__ fill, PBuf b) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n_ovf) return;
  const int k = key[e];
  if (k < 0) return;  // placed in a vacated slot
  const int slot = atomicAdd(fill + k, 1);
  copy_particle(b, e, b, pad + newb[k] + slot);
}

__global__ void __launch_bounds__(256) k_offset_copy(long long n, const int* __restrict__ src,
                                                     long long off, int* __restrict__ dst) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (int)(off + src[i]);
}

// Full deposition over the compact layout (CB: B^{n+1} from the centre stencil).
template <bool CB = false>
__global__ void __launch_bounds__(256) k_deposit(StepArgs a) {
  extern __shared__ __align__(16) float4 s_dyn[];
  constexpr int kDepSC = CB ? AMPS_CSC : AMPS_SC;
  float4* s_dep = s_dyn;
  float* s_rec = reinterpret_cast<float*>(s_dyn + kDepSC);
  __shared__ __align__(8) uint64_t bar;
  __shared__ double s_en[kWarps];
  const int b = blockIdx.x, k = blockIdx.y;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const void* src = CB ? (const void*)(a.st_ccur + (size_t)b * AMPS_CSC)
                       : (const void*)(a.st_dep + (size_t)b * AMPS_SC * AMPS_DEP_STRIDE);
  if (!stage_stencils(&bar, s_dep, src, kDepSC * 4 * sizeof(float), nullptr, nullptr, 0, a.flags))
    return;
  float* rec = s_rec + wid * kFields * kFS;
  int fA, fB;
  lane_fields(lane, fA, fB);
  FF en{0.f, 0.f};
  const int j = wid;
  const float inv_vol = block_inv_vol(a, b);
  for (int i = 0; i < AMPS_NC; i++) {
    const long long cid = (long long)b * AMPS_CPB + i + AMPS_NC * (j + AMPS_NC * k);
    const int b0 = a.base[cid], n0 = a.cnt[cid];
    Tile tile;
    tile.zero();
    for (int q0 = 0; q0 < n0; q0 += 32) {
      const long long p = b0 + q0 + lane;
      const bool act = q0 + lane < n0;
      // positions past the cell's particles stage zero weight at the cell centre
      float u[3] = {i + 0.5f, j + 0.5f, k + 0.5f}, v[3] = {0.f, 0.f, 0.f}, wq = 0.f;
      int s = 0;
      if (act) {
#pragma unroll
        for (int d = 0; d < 3; d++) { u[d] = a.p.u[d][p]; v[d] = a.p.v[d][p]; }
        s = a.p.sp[p];
        wq = a.p.wc ? a.p.wc[p] : 1.0f;
      }
      stage_fields<kFS, CB>(rec, lane, s_dep, u[0], u[1], u[2], v[0], v[1], v[2], s, wq, i, j, k,
                            a.st, inv_vol, en);
      __syncwarp();
      tile.accumulate<kFS>(rec, (min(32, n0 - q0) + 3) & ~3, fA, fB);
      __syncwarp();
    }
    tile.flush(lane, a.cellM, a.cellJ, cid);
  }
  reduce_energy(ff_value(en), s_en, a.energy);
}

// ---------------------------------------------------------------------------
// Corner assembly.  For corner c and each of its 8 cells, the pair (c, c2) of
// that cell lands in slot(c2 - c) of M_c; its block is the cell's partial of
// the pair's weight monomial.  The 64 (slot, cell, monomial) entries are
// grouped by slot so each output slot is written once.
struct AsmEntry {
  unsigned char slot, cell, mono, pad;
};
__constant__ AsmEntry c_asm[64];
__constant__ unsigned char c_asm_corner[8];

__global__ void __launch_bounds__(256) k_assemble(long long ncor, const int* __restrict__ nbr,
                                                  const float* __restrict__ cellM,
                                                  const float* __restrict__ cellJ, double inv_vol,
                                                  float* __restrict__ M, double* __restrict__ J) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncor) return;
  const int b = (int)(c / AMPS_CPB), l = (int)(c % AMPS_CPB);
  const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
  int cell[8];
#pragma unroll
  for (int co = 0; co < 8; co++)
    cell[co] = local_id(nbr, b, i - (co & 1), j - ((co >> 1) & 1), k - ((co >> 2) & 1));
  // sums of at most 8 FP32 partials per element (stored FP32)
  float acc[9];
  int cur = c_asm[0].slot;
#pragma unroll
  for (int e = 0; e < 9; e++) acc[e] = 0.f;
  for (int t = 0; t < 64; t++) {
    const AsmEntry en = c_asm[t];
    if (en.slot != cur) {
#pragma unroll
      for (int e = 0; e < 9; e++) {
        M[(size_t)(cur * 9 + e) * ncor + c] = acc[e];
        acc[e] = 0.f;
      }
      cur = en.slot;
    }
    const float* src = cellM + cellM_at(cell[en.cell], en.mono * 9);
#pragma unroll
    for (int e = 0; e < 9; e++) acc[e] += src[e];
  }
#pragma unroll
  for (int e = 0; e < 9; e++) M[(size_t)(cur * 9 + e) * ncor + c] = acc[e];
  float jj[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int co = 0; co < 8; co++) {
    const float* src = cellJ + cellJ_at(cell[co], c_asm_corner[co] * 3);
    jj[0] += src[0];
    jj[1] += src[1];
    jj[2] += src[2];
  }
  J[c] = widen(jj[0]) * inv_vol;
  J[ncor + c] = widen(jj[1]) * inv_vol;
  J[2 * ncor + c] = widen(jj[2]) * inv_vol;
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

// in and out may alias (each element is read before it is written by the same thread)
__global__ void __launch_bounds__(256) k_scan_final(const int* in, long long n,
                                                    const int* __restrict__ part, int* out) {
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
// Rebuild: unsorted particles (list buffer, keys) -> slotted layout.
__global__ void __launch_bounds__(256) k_rb_rank(long long n, const int* __restrict__ key,
                                                 int* __restrict__ rank, int* __restrict__ count) {
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n;
       base += (long long)gridDim.x * blockDim.x) {
    const long long p = base + threadIdx.x;
    // key < 0: deleted by the mover (open face), not placed
    const int k = p < n ? key[p] : -1;
    const bool act = k >= 0;
    const int r = warp_reserve(act, act ? k : 0, count);
    if (act) rank[p] = r;
  }
}

// cap[c] = count + slack, slack = count/4 + AMPS_SLACK_MIN scaled by num/den so
// that the total fits the slot capacity; cap[ncell] = 0 (scan terminator).
// The constant term keeps sparsely filled cells (fine AMR levels) from
// overflowing: a cell's occupancy random-walks by ~sqrt(2 x crossings) per
// step, and over 10^5 cells the largest excursion reaches ~4.5 of those.
__global__ void __launch_bounds__(256) k_rb_caps(long long ncell, const int* __restrict__ count,
                                                 int* __restrict__ cap, int num, int den) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c > ncell) return;
  if (c == ncell) { cap[c] = 0; return; }
  const int n = count[c];
  const int slack = (n >> 2) + AMPS_SLACK_MIN;
  cap[c] = n + (int)(((long long)slack * num) / den);
}

__global__ void __launch_bounds__(256) k_rb_scatter(long long n, const int* __restrict__ key,
                                                    const int* __restrict__ rank,
                                                    const int* __restrict__ base, PBuf s, PBuf d) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    const int k = key[p];
    if (k < 0) continue;  // deleted by the mover
    const long long q = (long long)base[k] + rank[p];
    copy_particle(s, p, d, q);
  }
}

// Append every particle of the compact layout to the list buffer (overflow
// recovery): one warp per cell, one atomic per chunk.
__global__ void __launch_bounds__(256) k_gather_valid(long long ncell, const int* __restrict__ base,
                                                      const int* __restrict__ cnt, PBuf s, PBuf d,
                                                      int* __restrict__ key,
                                                      unsigned long long* __restrict__ tail) {
  const long long cid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (cid >= ncell) return;
  const int b0 = base[cid], n0 = cnt[cid];
  for (int q0 = 0; q0 < n0; q0 += 32) {
    const int m = min(32, n0 - q0);
    unsigned long long o = 0;
    if (lane == 0) o = atomicAdd(tail, (unsigned long long)m);
    o = __shfl_sync(0xffffffffu, o, 0);
    if (lane < m) {
      copy_particle(s, b0 + q0 + lane, d, (long long)o + lane);
      key[o + lane] = (int)cid;
    }
  }
}

// ---------------------------------------------------------------------------
// Import: FP64 physical position -> block, cell, FP32 offset (findTreeNode +
// FindCellIndex + periodic exchange rules) into the unsorted list buffer.
struct ImportArgs {
  const double* x; const double* v; const uint8_t* sp; const double* wc;
  PBuf d;
  int* key;
  unsigned long long* flags;
  long long n;
  int nbk[3];
  double x0[3], dx[3];
  int nspec;
};

__global__ void __launch_bounds__(256) k_import(ImportArgs a) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < a.n;
       p += (long long)gridDim.x * blockDim.x) {
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
        const int br = ((bb % a.nbk[d]) + a.nbk[d]) % a.nbk[d];
        const double xr = a.x0[d] + br * L;
        x += xr - xmin;
        if (x < xr) x = xr;
        if (x >= xr + L) x = (xr + L) - 1.0E-10 * L;
        bb = br;
        xmin = xr;
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
    a.key[p] = blk * AMPS_CPB + ic[0] + AMPS_NC * (ic[1] + AMPS_NC * ic[2]);
    for (int d = 0; d < 3; d++) {
      a.d.u[d][p] = uf[d];
      a.d.v[d][p] = (float)a.v[3 * p + d];
    }
    const int s = a.sp[p];
    if (s >= a.nspec) atomicAdd(a.flags + 2, 1ull);
    a.d.sp[p] = (uint8_t)s;
    if (a.d.wc) a.d.wc[p] = a.wc ? (float)a.wc[p] : 1.0f;
    if (a.d.id) a.d.id[p] = (uint32_t)p;
  }
}

// AMR import: FP64 position -> leaf block through the finest-block map, cell
// and FP32 offset in that block's cell units (same periodic rules).
struct ImportAmrArgs {
  const double* x; const double* v; const uint8_t* sp; const double* wc;
  PBuf d;
  int* key;
  unsigned long long* flags;
  long long n;
  AmrDev m;
  double x0[3], dxf;
  int nspec;
};

__global__ void __launch_bounds__(256) k_import_amr(ImportAmrArgs a) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < a.n;
       p += (long long)gridDim.x * blockDim.x) {
    double x[3];
    int F[3];
    for (int d = 0; d < 3; d++) {
      const double L = a.m.nfine[d] * a.dxf;
      double xx = a.x[3 * p + d];
      if (xx < a.x0[d]) xx += L;
      if (xx >= a.x0[d] + L) xx -= L;
      if (xx >= a.x0[d] + L) xx = a.x0[d] + L - 1e-10 * a.dxf;
      if (xx < a.x0[d]) xx = a.x0[d];
      int f = (int)floor((xx - a.x0[d]) / a.dxf);
      F[d] = min(max(f, 0), a.m.nfine[d] - 1);
      x[d] = xx;
    }
    const int nb0 = a.m.nfine[0] >> 3, nb1 = a.m.nfine[1] >> 3;
    const int blk = a.m.fine_map[(F[0] >> 3) + nb0 * ((F[1] >> 3) + nb1 * (F[2] >> 3))];
    const double dx = a.m.bscale[blk] * a.dxf;
    int ic[3];
    for (int d = 0; d < 3; d++) {
      const double o = a.x0[d] + a.m.borg[3 * blk + d] * a.dxf;
      const double ud = (x[d] - o) / dx;
      int ci = (int)ud;
      if (ci >= AMPS_NC) ci = AMPS_NC - 1;
      if (ci < 0) ci = 0;
      float u = (float)ud;
      if (u < (float)ci) u = (float)ci;
      if (u >= (float)(ci + 1)) u = nextafterf((float)(ci + 1), 0.0f);
      ic[d] = ci;
      a.d.u[d][p] = u;
      a.d.v[d][p] = (float)a.v[3 * p + d];
    }
    a.key[p] = blk * AMPS_CPB + ic[0] + AMPS_NC * (ic[1] + AMPS_NC * ic[2]);
    const int s = a.sp[p];
    if (s >= a.nspec) atomicAdd(a.flags + 2, 1ull);
    a.d.sp[p] = (uint8_t)s;
    if (a.d.wc) a.d.wc[p] = a.wc ? (float)a.wc[p] : 1.0f;
    if (a.d.id) a.d.id[p] = (uint32_t)p;
  }
}

// Local import: interleaved FP32 offsets/velocities and block ids.
__global__ void __launch_bounds__(256) k_import_local(long long n, const float* __restrict__ u,
                                                      const float* __restrict__ v,
                                                      const uint8_t* __restrict__ sp,
                                                      const int* __restrict__ blk,
                                                      const float* __restrict__ wc, int nb,
                                                      int nspec, PBuf d, int* key,
                                                      unsigned long long* flags) {
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < n;
       p += (long long)gridDim.x * blockDim.x) {
    int ic[3];
    for (int q = 0; q < 3; q++) {
      float uu = u[3 * p + q];
      if (!(uu >= 0.f && uu < 8.f)) atomicAdd(flags + 2, 1ull);
      uu = clamp_below8(fmaxf(uu, 0.f));
      ic[q] = min((int)uu, AMPS_NC - 1);
      d.u[q][p] = uu;
      d.v[q][p] = v[3 * p + q];
    }
    int b = blk[p];
    if (b < 0 || b >= nb) { atomicAdd(flags + 2, 1ull); b = 0; }
    const int s = sp[p];
    if (s >= nspec) atomicAdd(flags + 2, 1ull);
    d.sp[p] = (uint8_t)s;
    if (d.wc) d.wc[p] = wc ? wc[p] : 1.0f;
    if (d.id) d.id[p] = (uint32_t)p;
    key[p] = b * AMPS_CPB + ic[0] + AMPS_NC * (ic[1] + AMPS_NC * ic[2]);
  }
}

// Export: compact arrays in cell order (out offsets = exclusive scan of cnt).
__global__ void __launch_bounds__(256) k_export(long long ncells, const int* __restrict__ base,
                                                const int* __restrict__ cnt,
                                                const int* __restrict__ out0, PBuf s, int nbx,
                                                int nby, double x00, double x01, double x02,
                                                double dx0, double dx1, double dx2, double* x,
                                                double* v, uint8_t* sp, int32_t* blk,
                                                int32_t* cel, uint32_t* id, AmrDev m, double dxf) {
  const long long cid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cid >= ncells) return;
  const int b = (int)(cid / AMPS_CPB), l = (int)(cid % AMPS_CPB);
  double o0, o1, o2;
  if (m.borg) {
    // AMR: origin on the finest lattice, cell size a power of two of the finest
    o0 = x00 + m.borg[3 * b] * dxf;
    o1 = x01 + m.borg[3 * b + 1] * dxf;
    o2 = x02 + m.borg[3 * b + 2] * dxf;
    dx0 = dx1 = dx2 = m.bscale[b] * dxf;
  } else {
    const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
    o0 = x00 + bx * (AMPS_NC * dx0);
    o1 = x01 + by * (AMPS_NC * dx1);
    o2 = x02 + bz * (AMPS_NC * dx2);
  }
  const int b0 = base[cid], n0 = cnt[cid];
  long long q = out0[cid];
  for (int t = 0; t < n0; t++, q++) {
    const long long p = b0 + t;
    if (x) {
      x[3 * q] = o0 + (double)s.u[0][p] * dx0;
      x[3 * q + 1] = o1 + (double)s.u[1][p] * dx1;
      x[3 * q + 2] = o2 + (double)s.u[2][p] * dx2;
    }
    if (v) {
      v[3 * q] = s.v[0][p];
      v[3 * q + 1] = s.v[1][p];
      v[3 * q + 2] = s.v[2][p];
    }
    if (sp) sp[q] = s.sp[p];
    if (blk) blk[q] = b;
    if (cel) cel[q] = l;
    if (id && s.id) id[q] = s.id[p];
  }
}

// ---------------------------------------------------------------------------
// Mover::Relativistic::Boris (src/pic/pic_mover_relativistic_boris.cpp:16-583,
// scalar path :119-175) on the mesh: FP64 sub-steps of dt = min(1/f_g,
// remaining), f_g = |q||B|/(2 pi m gamma) (specfunc.h:1290), fields E, B
// interpolated from the FP64 corner arrays at each sub-step's start position
// (CornerBased::InitStencil weights, normalised), periodic re-location after
// every sub-step (findTreeNode rules).  One thread per particle of the list
// buffer; writes the new block-local offset, velocity and key.
struct RelBorisArgs {
  PBuf d;
  int* key;
  long long n;
  const int* nbr;
  long long ncor;
  const double* E;
  const double* B;
  int nbk[3];
  double x0[3], dx[3];
  double qm[AMPS_GPU_MAX_SPECIES];  // q/m per species
  double qabs_over_m[AMPS_GPU_MAX_SPECIES];
  double dt_total, c_light;
  long long max_sub;
  unsigned long long* flags;   // [2] sub-step cap reached, [6] deleted at an open face
  unsigned long long* nsub;    // total sub-steps
  int open;                    // bit d: axis d open (a particle past its faces is deleted)
};

// block and in-block coordinate of x (periodic; same rules as k_import)
__device__ __forceinline__ void rb_locate(const RelBorisArgs& a, double x[3], int bx[3],
                                          double xmin[3]) {
  for (int d = 0; d < 3; d++) {
    const double L = AMPS_NC * a.dx[d];
    int bb = (int)floor((x[d] - a.x0[d]) / L);
    double xm = a.x0[d] + bb * L;
    if (x[d] < xm) { bb--; xm = a.x0[d] + bb * L; }
    if (x[d] >= xm + L) { bb++; xm = a.x0[d] + bb * L; }
    if (bb < 0 || bb >= a.nbk[d]) {
      const int br = ((bb % a.nbk[d]) + a.nbk[d]) % a.nbk[d];
      const double xr = a.x0[d] + br * L;
      x[d] += xr - xm;
      if (x[d] < xr) x[d] = xr;
      if (x[d] >= xr + L) x[d] = (xr + L) - 1.0E-10 * L;
      bb = br;
      xm = xr;
    }
    bx[d] = bb;
    xmin[d] = xm;
  }
}

// Mover::Boris (src/pic/pic_mover_boris.cpp:126-553, scalar path :264-290)
// with BorisSplitAcceleration_default's Lorentz force (:104-112): one step of
// dt_total, u = v + dt/2 (q/m) E, h = dt/2 (q/m) B, U = ((1-h^2) u + 2 (u x h
// + (u.h) h)) / (1+h^2), v' = U + dt/2 (q/m) E, x' = x + dt v'.
__device__ __forceinline__ void boris_plain(double qm, double dt, const double Ef[3],
                                            const double Bf[3], double v[3]) {
  const double dt2 = dt / 2.0;
  double accl[3], u[3], h[3];
  for (int d = 0; d < 3; d++) {
    accl[d] = qm * Ef[d];
    u[d] = v[d] + dt2 * accl[d];
    h[d] = -dt2 * (-(qm * Bf[d]));
  }
  const double h2 = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
  const double uh = u[0] * h[0] + u[1] * h[1] + u[2] * h[2];
  const double U0 = ((1 - h2) * u[0] + 2 * (u[1] * h[2] - h[1] * u[2] + uh * h[0])) / (1 + h2);
  const double U1 = ((1 - h2) * u[1] + 2 * (u[2] * h[0] - h[2] * u[0] + uh * h[1])) / (1 + h2);
  const double U2 = ((1 - h2) * u[2] + 2 * (u[0] * h[1] - h[0] * u[1] + uh * h[2])) / (1 + h2);
  v[0] = U0 + dt2 * accl[0];
  v[1] = U1 + dt2 * accl[1];
  v[2] = U2 + dt2 * accl[2];
}

// REL: Mover::Relativistic::Boris with gyro-period sub-steps; !REL: one plain
// Boris step of dt_total (fields and re-location as above).
template <bool REL>
__global__ void __launch_bounds__(256) k_relboris(RelBorisArgs a) {
  unsigned long long my_sub = 0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < a.n;
       p += (long long)gridDim.x * blockDim.x) {
    const int key = a.key[p];
    const int b0 = key / AMPS_CPB;
    const int sp = a.d.sp[p];
    int bx[3] = {b0 % a.nbk[0], (b0 / a.nbk[0]) % a.nbk[1], b0 / (a.nbk[0] * a.nbk[1])};
    double x[3], v[3];
    for (int d = 0; d < 3; d++) {
      x[d] = a.x0[d] + bx[d] * (AMPS_NC * a.dx[d]) + (double)a.d.u[d][p] * a.dx[d];
      v[d] = a.d.v[d][p];
    }
    double rem = a.dt_total;
    long long ns = 0;
    double xmin[3];
    while (rem > 0.0) {
      if (ns >= a.max_sub) {
        atomicAdd(a.flags + 2, 1ull);
        break;
      }
      rb_locate(a, x, bx, xmin);
      const int b = bx[0] + a.nbk[0] * (bx[1] + a.nbk[1] * bx[2]);
      int iX[3];
      double xl[3];
      for (int d = 0; d < 3; d++) {
        const double xmax = xmin[d] + AMPS_NC * a.dx[d];
        double xx = x[d];
        if (fabs(xx - xmax) < 1e-10 * a.dx[d]) xx = xmax - 1e-10 * a.dx[d];
        xl[d] = (xx - xmin[d]) / a.dx[d];
        iX[d] = min(max((int)xl[d], 0), AMPS_NC - 1);
        xl[d] -= iX[d];
      }
      double w[8], norm = 0.0;
      for (int q = 0; q < 8; q++) {
        const int aa = q & 1, bb = (q >> 1) & 1, cc = q >> 2;
        w[q] = (aa ? xl[0] : 1.0 - xl[0]) * (bb ? xl[1] : 1.0 - xl[1]) * (cc ? xl[2] : 1.0 - xl[2]);
        norm += w[q];
      }
      double Ef[3] = {0, 0, 0}, Bf[3] = {0, 0, 0};
      for (int q = 0; q < 8; q++) {
        const int id = local_id(a.nbr, b, iX[0] + (q & 1), iX[1] + ((q >> 1) & 1), iX[2] + (q >> 2));
        const double wq = w[q] / norm;
        for (int d = 0; d < 3; d++) {
          Ef[d] += wq * a.E[d * a.ncor + id];
          Bf[d] += wq * a.B[d * a.ncor + id];
        }
      }
      if (!REL) {
        const double dt = rem;
        rem = 0.0;
        boris_plain(a.qm[sp], dt, Ef, Bf, v);
        for (int d = 0; d < 3; d++) {
          x[d] += dt * v[d];
          if (((a.open >> d) & 1) && (x[d] < a.x0[d] || x[d] >= a.x0[d] + a.nbk[d] * AMPS_NC * a.dx[d]))
            rem = -1.0;
        }
        ns++;
        continue;
      }
      const double cc2 = a.c_light * a.c_light;
      double gam = 1.0 / sqrt(1.0 - (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / cc2);
      const double bmag = sqrt(Bf[0] * Bf[0] + Bf[1] * Bf[1] + Bf[2] * Bf[2]);
      double dt = rem;
      if (bmag > 1.0e-25) {
        const double fg = a.qabs_over_m[sp] * bmag / (2.0 * 3.14159265358979323846 * gam);
        const double dtmax = 1.0 / fg;
        if (dtmax < rem) dt = dtmax;
      }
      rem -= dt;
      const double h = 0.5 * a.qm[sp] * dt;
      double um[3], t[3], up[3], sv[3], upl[3], uf[3], l = 0.0;
      for (int d = 0; d < 3; d++) um[d] = gam * v[d] + h * Ef[d];
      gam = sqrt(1.0 + (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]) / cc2);
      for (int d = 0; d < 3; d++) { t[d] = h / gam * Bf[d]; l += t[d] * t[d]; }
      up[0] = um[0] + (um[1] * t[2] - um[2] * t[1]);
      up[1] = um[1] + (um[2] * t[0] - um[0] * t[2]);
      up[2] = um[2] + (um[0] * t[1] - um[1] * t[0]);
      for (int d = 0; d < 3; d++) sv[d] = 2.0 * t[d] / (1.0 + l);
      upl[0] = um[0] + (up[1] * sv[2] - up[2] * sv[1]);
      upl[1] = um[1] + (up[2] * sv[0] - up[0] * sv[2]);
      upl[2] = um[2] + (up[0] * sv[1] - up[1] * sv[0]);
      for (int d = 0; d < 3; d++) uf[d] = upl[d] + h * Ef[d];
      gam = sqrt(1.0 + (uf[0] * uf[0] + uf[1] * uf[1] + uf[2] * uf[2]) / cc2);
      for (int d = 0; d < 3; d++) {
        v[d] = uf[d] / gam;
        x[d] += v[d] * dt;
        if (((a.open >> d) & 1) && (x[d] < a.x0[d] || x[d] >= a.x0[d] + a.nbk[d] * AMPS_NC * a.dx[d]))
          rem = -1.0;
      }
      ns++;
    }
    my_sub += (unsigned long long)ns;
    if (rem < 0.0) {  // left the domain through an open face
      a.key[p] = -1;
      atomicAdd(a.flags + 6, 1ull);
      continue;
    }
    // final block, cell and FP32 offset
    rb_locate(a, x, bx, xmin);
    int ic[3];
    for (int d = 0; d < 3; d++) {
      int ci = (int)((x[d] - xmin[d]) / a.dx[d]);
      ci = min(max(ci, 0), AMPS_NC - 1);
      float u = (float)((x[d] - xmin[d]) / a.dx[d]);
      if (u < (float)ci) u = (float)ci;
      if (u >= (float)(ci + 1)) u = nextafterf((float)(ci + 1), 0.0f);
      ic[d] = ci;
      a.d.u[d][p] = u;
      a.d.v[d][p] = (float)v[d];
    }
    const int blk = bx[0] + a.nbk[0] * (bx[1] + a.nbk[1] * bx[2]);
    a.key[p] = blk * AMPS_CPB + ic[0] + AMPS_NC * (ic[1] + AMPS_NC * ic[2]);
  }
  if (my_sub) atomicAdd(a.nsub, my_sub);
}

// The same mover on a periodic AMR mesh (block tree of AmrDev): at the start
// of every sub-step the particle is re-located (periodic wrap, finest-block
// map: k_import_amr's rules) and E, B are interpolated from that leaf block's
// 8 cell corners (FP64 component-major corner arrays over the unique corners;
// a hanging corner takes its constraint P, CSR hs/hp/hw).  The sub-step rule
// and the update are k_relboris's.
struct AmrRelBorisArgs {
  PBuf d;
  int* key;
  long long n;
  AmrDev m;
  const int* ctab;
  const int* hs;
  const int* hp;
  const double* hw;
  long long nvc;
  const double* E;
  const double* B;
  double x0[3], dxf;
  double qm[AMPS_GPU_MAX_SPECIES];
  double qabs_over_m[AMPS_GPU_MAX_SPECIES];
  double dt_total, c_light;
  long long max_sub;
  unsigned long long* flags;
  unsigned long long* nsub;
  int open;
};

__device__ __forceinline__ int amr_rb_locate(const AmrRelBorisArgs& a, double x[3]) {
  int F[3];
  for (int d = 0; d < 3; d++) {
    const double L = a.m.nfine[d] * a.dxf;
    // a sub-step can carry a fast particle more than one period
    const double k = floor((x[d] - a.x0[d]) / L);
    if (k != 0.0) x[d] -= k * L;
    if (x[d] < a.x0[d]) x[d] += L;
    if (x[d] >= a.x0[d] + L) x[d] -= L;
    if (x[d] >= a.x0[d] + L) x[d] = a.x0[d] + L - 1e-10 * a.dxf;
    if (x[d] < a.x0[d]) x[d] = a.x0[d];
    F[d] = min(max((int)floor((x[d] - a.x0[d]) / a.dxf), 0), a.m.nfine[d] - 1);
  }
  const int nb0 = a.m.nfine[0] >> 3, nb1 = a.m.nfine[1] >> 3;
  return a.m.fine_map[(F[0] >> 3) + nb0 * ((F[1] >> 3) + nb1 * (F[2] >> 3))];
}

template <bool REL>
__global__ void __launch_bounds__(256) k_amr_relboris(AmrRelBorisArgs a) {
  unsigned long long my_sub = 0;
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < a.n;
       p += (long long)gridDim.x * blockDim.x) {
    int blk = a.key[p] / AMPS_CPB;
    const int sp = a.d.sp[p];
    double x[3], v[3];
    for (int d = 0; d < 3; d++) {
      x[d] = a.x0[d] + a.m.borg[3 * blk + d] * a.dxf + (double)a.d.u[d][p] * (a.m.bscale[blk] * a.dxf);
      v[d] = a.d.v[d][p];
    }
    const double cc2 = a.c_light * a.c_light;
    double rem = a.dt_total;
    long long ns = 0;
    while (rem > 0.0) {
      if (ns >= a.max_sub) {
        atomicAdd(a.flags + 2, 1ull);
        break;
      }
      blk = amr_rb_locate(a, x);
      const double dx = a.m.bscale[blk] * a.dxf;
      int ic[3];
      double f[3];
      for (int d = 0; d < 3; d++) {
        const double u = (x[d] - (a.x0[d] + a.m.borg[3 * blk + d] * a.dxf)) / dx;
        ic[d] = min(max((int)u, 0), AMPS_NC - 1);
        f[d] = u - ic[d];
      }
      double Ef[3] = {0, 0, 0}, Bf[3] = {0, 0, 0};
#pragma unroll 1
      for (int q = 0; q < 8; q++) {
        // table order (0,0,0) (1,0,0) (1,1,0) (0,1,0) (0,0,1) (1,0,1) (1,1,1) (0,1,1)
        const int ox = ((q + 1) >> 1) & 1, oy = (q >> 1) & 1, oz = q >> 2;
        const double w = 1.0 * (ox ? f[0] : 1.0 - f[0]) * (oy ? f[1] : 1.0 - f[1]) * (oz ? f[2] : 1.0 - f[2]);
        const int cc = a.ctab[blk * 729 + (ic[0] + ox) + 9 * ((ic[1] + oy) + 9 * (ic[2] + oz))];
        const int hs0 = a.hs[cc], hs1 = a.hs[cc + 1];
        for (int d = 0; d < 3; d++) {
          double e, b;
          if (hs0 == hs1) {
            e = a.E[d * a.nvc + cc];
            b = a.B[d * a.nvc + cc];
          } else {
            e = 0.0;
            b = 0.0;
            for (int t = hs0; t < hs1; t++) {
              e += a.hw[t] * a.E[d * a.nvc + a.hp[t]];
              b += a.hw[t] * a.B[d * a.nvc + a.hp[t]];
            }
          }
          Ef[d] += w * e;
          Bf[d] += w * b;
        }
      }
      if (!REL) {
        const double dt = rem;
        rem = 0.0;
        boris_plain(a.qm[sp], dt, Ef, Bf, v);
        for (int d = 0; d < 3; d++) {
          x[d] += dt * v[d];
          if (((a.open >> d) & 1) && (x[d] < a.x0[d] || x[d] >= a.x0[d] + a.m.nfine[d] * a.dxf))
            rem = -1.0;
        }
        ns++;
        continue;
      }
      double gam = 1.0 / sqrt(1.0 - (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / cc2);
      const double bmag = sqrt(Bf[0] * Bf[0] + Bf[1] * Bf[1] + Bf[2] * Bf[2]);
      double dt = rem;
      if (bmag > 1.0e-25) {
        const double dtmax = 1.0 / (a.qabs_over_m[sp] * bmag / (2.0 * 3.14159265358979323846 * gam));
        if (dtmax < rem) dt = dtmax;
      }
      rem -= dt;
      const double h = 0.5 * a.qm[sp] * dt;
      double um[3], t[3], up[3], sv[3], upl[3], uf[3], l = 0.0;
      for (int d = 0; d < 3; d++) um[d] = gam * v[d] + h * Ef[d];
      gam = sqrt(1.0 + (um[0] * um[0] + um[1] * um[1] + um[2] * um[2]) / cc2);
      for (int d = 0; d < 3; d++) { t[d] = h / gam * Bf[d]; l += t[d] * t[d]; }
      up[0] = um[0] + (um[1] * t[2] - um[2] * t[1]);
      up[1] = um[1] + (um[2] * t[0] - um[0] * t[2]);
      up[2] = um[2] + (um[0] * t[1] - um[1] * t[0]);
      for (int d = 0; d < 3; d++) sv[d] = 2.0 * t[d] / (1.0 + l);
      upl[0] = um[0] + (up[1] * sv[2] - up[2] * sv[1]);
      upl[1] = um[1] + (up[2] * sv[0] - up[0] * sv[2]);
      upl[2] = um[2] + (up[0] * sv[1] - up[1] * sv[0]);
      for (int d = 0; d < 3; d++) uf[d] = upl[d] + h * Ef[d];
      gam = sqrt(1.0 + (uf[0] * uf[0] + uf[1] * uf[1] + uf[2] * uf[2]) / cc2);
      for (int d = 0; d < 3; d++) {
        v[d] = uf[d] / gam;
        x[d] += v[d] * dt;
        if (((a.open >> d) & 1) && (x[d] < a.x0[d] || x[d] >= a.x0[d] + a.m.nfine[d] * a.dxf))
          rem = -1.0;
      }
      ns++;
    }
    my_sub += (unsigned long long)ns;
    if (rem < 0.0) {  // left the domain through an open face
      a.key[p] = -1;
      atomicAdd(a.flags + 6, 1ull);
      continue;
    }
    // final leaf block, cell and FP32 offset (k_import_amr's rules)
    blk = amr_rb_locate(a, x);
    const double dx = a.m.bscale[blk] * a.dxf;
    int ic[3];
    for (int d = 0; d < 3; d++) {
      const double ud = (x[d] - (a.x0[d] + a.m.borg[3 * blk + d] * a.dxf)) / dx;
      const int ci = min(max((int)ud, 0), AMPS_NC - 1);
      float u = (float)ud;
      if (u < (float)ci) u = (float)ci;
      if (u >= (float)(ci + 1)) u = nextafterf((float)(ci + 1), 0.0f);
      ic[d] = ci;
      a.d.u[d][p] = u;
      a.d.v[d][p] = (float)v[d];
    }
    a.key[p] = blk * AMPS_CPB + ic[0] + AMPS_NC * (ic[1] + AMPS_NC * ic[2]);
  }
  if (my_sub) atomicAdd(a.nsub, my_sub);
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
      // cell = corner - (co&1, (co>>1)&1, (co>>2)&1): the corner sits at local
      // offset (co&1, (co>>1)&1, (co>>2)&1) of that cell
      const int lx = co & 1, ly = (co >> 1) & 1, lz = (co >> 2) & 1;
      const int c1 = tidx(lx, ly, lz);
      corner_of[co] = (unsigned char)c1;
      for (int c2 = 0; c2 < 8; c2++) {
        const int ddx = off[c2][0] - lx, ddy = off[c2][1] - ly, ddz = off[c2][2] - lz;
        if (mm_slot(ddx, ddy, ddz) != slot) continue;
        e[n].slot = (unsigned char)slot;
        e[n].cell = (unsigned char)co;
        e[n].mono = (unsigned char)pair_monomial(c1, c2);
        e[n].pad = 0;
        n++;
      }
    }
  cudaMemcpyToSymbol(c_asm, e, sizeof(e));
  cudaMemcpyToSymbol(c_asm_corner, corner_of, sizeof(corner_of));
  g_asm_ready = true;
}

StepArgs step_args(amps_gpu_ctx* c) {
  StepArgs a;
  a.nbr = c->d_nbr;
  a.base = c->d_base;
  a.cnt = c->d_cnt;
  a.arr = c->d_arr;
  a.stay = c->d_stay;
  a.st_push = c->d_stencil_push;
  a.st_dep = c->d_stencil_dep;
  a.st_cprev = c->b_center ? reinterpret_cast<const float4*>(c->d_stencil_cprev) : nullptr;
  a.st_ccur = c->b_center ? reinterpret_cast<const float4*>(c->d_stencil_ccur) : nullptr;
  a.p = pbuf(c, c->cur);
  a.ovf = pbuf(c, c->cur ^ 1);
  a.ovf_key = c->d_key;
  a.cellM = c->d_cellM;
  a.cellJ = c->d_cellJ;
  a.energy = c->d_energy;
  a.flags = c->d_flags;
  for (int d = 0; d < 3; d++) a.dtdx[d] = (float)(c->cfg.dt / c->cfg.dx[d]);
  a.inv_vol = (float)(1.0 / (c->cfg.dx[0] * c->cfg.dx[1] * c->cfg.dx[2]));
  a.ovf_cap = c->slots;
  a.st = make_species(c->cfg);
  a.amr = c->amrdev;
  a.open = c->open_axes;
  a.nbk[0] = c->cfg.nbx;
  a.nbk[1] = c->cfg.nby;
  a.nbk[2] = c->cfg.nbz;
  return a;
}

size_t smem_push(bool dep, bool cb = false) {
  return (size_t)(2 * AMPS_SC + (cb ? 2 * AMPS_CSC : AMPS_SC)) * sizeof(float4) +
         (dep ? kWarps * kFields * kFS * sizeof(float) : 0);
}
size_t smem_dep(bool cb = false) {
  return (size_t)(cb ? AMPS_CSC : AMPS_SC) * sizeof(float4) + kWarps * kFields * kFS * sizeof(float);
}
size_t smem_arr(int chunk) { return (size_t)kWarps * kFields * (chunk + 4) * sizeof(float); }

void set_smem_attrs() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(k_push_deposit<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_push(true));
  cudaFuncSetAttribute(k_push_deposit<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_push(false));
  cudaFuncSetAttribute(k_push_deposit<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_push(true));
  cudaFuncSetAttribute(k_push_deposit<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_push(false));
  cudaFuncSetAttribute(k_arrivals<true, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_arr(16));
  cudaFuncSetAttribute(k_arrivals<false, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_arr(16));
  cudaFuncSetAttribute(k_arrivals<true, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_arr(32));
  cudaFuncSetAttribute(k_arrivals<false, 32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_arr(32));
  cudaFuncSetAttribute(k_deposit<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_dep(false));
  cudaFuncSetAttribute(k_deposit<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_dep(true));
  cudaFuncSetAttribute(k_push_deposit<true, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem_push(true, true));
  cudaFuncSetAttribute(k_push_deposit<false, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem_push(false, true));
  cudaFuncSetAttribute(k_arrivals<true, 16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_arr(16));
  cudaFuncSetAttribute(k_arrivals<false, 16, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_arr(16));
  cudaFuncSetAttribute(k_arrivals<true, 32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_arr(32));
  cudaFuncSetAttribute(k_arrivals<false, 32, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_arr(32));
  done = true;
}

cudaError_t scan_ints(amps_gpu_ctx* c, const int* in, int* out, long long n) {
  const int tiles = (int)((n + kScanTile - 1) / kScanTile);
  TimedLaunch t(c, "scan", 3);
  k_scan_reduce<<<tiles, 256, 0, c->stream>>>(in, n, c->d_scan_part);
  k_scan_parts<<<1, 1024, 0, c->stream>>>(c->d_scan_part, tiles);
  k_scan_final<<<tiles, 256, 0, c->stream>>>(in, n, c->d_scan_part, out);
  return cudaGetLastError();
}

}  // namespace

// Counting sort of the list buffer (cur^1, keys in d_key) with n particles into
// the slotted layout of buffer cur.
cudaError_t rebuild_from_list(amps_gpu_ctx* c, long long n) {
  cudaStream_t s = c->stream;
  const long long nc = c->ncor;
  cudaError_t e = cudaMemsetAsync(c->d_count, 0, sizeof(int) * (nc + 1), s);
  if (e != cudaSuccess) return e;
  {
    TimedLaunch t(c, "rebuild");
    k_rb_rank<<<grid_for(n, 256), 256, 0, s>>>(n, c->d_key, c->d_rank, c->d_count);
  }
  return place_ranked(c, n);
}

// Second half of the counting sort: d_count holds the per-cell counts and
// d_key/d_rank each list entry's cell and rank in it; lays out buffer cur with
// slack and scatters the list buffer (cur^1) into it.  The restart reader
// fills the ranks itself, so that each cell keeps the list order of the file.
cudaError_t place_ranked(amps_gpu_ctx* c, long long n) {
  cudaStream_t s = c->stream;
  const long long nc = c->ncor;
  cudaError_t e;
  // slack scaled so that sum(cap) <= slots: sum(cap) <= n + n/4 + AMPS_SLACK_MIN nc
  const long long worst = n + n / 4 + (long long)AMPS_SLACK_MIN * nc;
  int num = 1, den = 1;
  if (worst > c->slots) {
    num = (int)std::max(0LL, (c->slots - n) / 1024);
    den = (int)std::max(1LL, (worst - n) / 1024 + 1);
  }
  {
    TimedLaunch t(c, "rebuild");
    k_rb_caps<<<(unsigned)((nc + 1 + 255) / 256), 256, 0, s>>>(nc, c->d_count, c->d_tmp, num, den);
  }
  e = scan_ints(c, c->d_tmp, c->d_base, nc + 1);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(c->d_sp[c->cur], 0xFF, (size_t)c->slots, s);
  if (e != cudaSuccess) return e;
  {
    TimedLaunch t(c, "rebuild");
    k_rb_scatter<<<grid_for(n, 256), 256, 0, s>>>(n, c->d_key, c->d_rank, c->d_base,
                                                   pbuf(c, c->cur ^ 1), pbuf(c, c->cur));
  }
  e = cudaMemcpyAsync(c->d_cnt, c->d_count, sizeof(int) * nc, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return e;
  return cudaMemsetAsync(c->d_arr, 0, sizeof(int) * nc, s);
}

// ===========================================================================
// launchers

// one-time host-side setup of the particle kernels (kernel attributes, the
// constant assembly table); must precede any stream capture
void particles_prepare() {
  set_smem_attrs();
  init_asm_table();
}

cudaError_t launch_pack_stencils(amps_gpu_ctx* c, const double* Eh, const double* Bprev,
                                 const double* Bcur) {
  if (c->amr) return launch_amr_pack(c, Eh, Bprev, Bcur);
  TimedLaunch t(c, "pack_stencils");
  // centre B: B^n in the scratch slot d_Bc2 (the field solve swaps it there;
  // the field import copies the imported centres into it), B^{n+1} in d_Bc
  const bool cb = c->b_center;
  k_pack_stencils<<<c->nb, 256, 0, c->stream>>>(
      c->nb, c->ncor, c->d_nbr, Eh, Bprev, Bcur, c->d_stencil_push, c->d_stencil_dep,
      cb ? c->d_Bc2 : nullptr, cb ? c->d_Bc : nullptr,
      cb ? reinterpret_cast<float4*>(c->d_stencil_cprev) : nullptr,
      cb ? reinterpret_cast<float4*>(c->d_stencil_ccur) : nullptr);
  return cudaGetLastError();
}

// On AMR meshes the field operator reads the per-cell partials directly.
static cudaError_t launch_assemble(amps_gpu_ctx* c) {
  if (c->amr) return cudaSuccess;
  init_asm_table();
  TimedLaunch t(c, "assemble");
  const double inv_vol = 1.0 / (c->cfg.dx[0] * c->cfg.dx[1] * c->cfg.dx[2]);
  k_assemble<<<(unsigned)((c->ncor + 255) / 256), 256, 0, c->stream>>>(
      c->ncor, c->d_nbr, c->d_cellM, c->d_cellJ, inv_vol, c->d_M, c->d_J);
  return cudaGetLastError();
}

// Full deposit (UpdateJMassMatrix on the current layout).
cudaError_t launch_deposit(amps_gpu_ctx* c) {
  set_smem_attrs();
  cudaError_t e = cudaMemsetAsync(c->d_energy, 0, sizeof(double), c->stream);
  if (e != cudaSuccess) return e;
  StepArgs a = step_args(c);
  {
    TimedLaunch t(c, "deposit");
    if (c->b_center)
      k_deposit<true><<<dim3(c->nb, AMPS_NC), kWarps * 32, smem_dep(true), c->stream>>>(a);
    else
      k_deposit<false><<<dim3(c->nb, AMPS_NC), kWarps * 32, smem_dep(false), c->stream>>>(a);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_assemble(c);
}

// Push (+ deposit) of one step: k_push_deposit, k_arrivals (+ assemble).
// Overflow recovery is done by the caller (particles_place_overflow,
// particles_relayout).
// ids of injected particles continue after the imported ones (0..n-1)
void set_next_id(amps_gpu_ctx* c, long long n) {
  c->next_id = (uint32_t)n;
  if (c->d_step) k_set_next_id<<<1, 32, 0, c->stream>>>(c->d_step, (unsigned long long)n);
}

// CalculateInjectionRate_MaxwellianDistribution (src/pic/pic_bc.cpp:215-242):
// number flux through a face of outward normal n of a Maxwellian with number
// density, bulk velocity and beta = 1 / (sqrt(2) vth)
static double maxwellian_flux(double density, const double drift[3], double beta, const double n[3]) {
  const double kSqrtPi = 1.7724538509055160273;
  double vv = 0.0, vnorm = 0.0;
  for (int d = 0; d < 3; d++) {
    vv += drift[d] * drift[d];
    vnorm += drift[d] * n[d];
  }
  vv = std::sqrt(vv);
  const double sc = vv * beta;
  if (sc > 10.0 && vnorm < 0.0) return std::fabs(vnorm) * density;
  if (sc > 10.0 && vnorm > 0.0) return 0.0;
  double aa;
  if (vv > 1.0e-6) {
    const double cc = -vnorm / vv;
    aa = (std::exp(-sc * sc * cc * cc) + kSqrtPi * sc * cc * (1.0 + std::erf(sc * cc))) / (2.0 * kSqrtPi);
  } else {
    aa = 1.0 / (2.0 * kSqrtPi);
  }
  return std::fabs(aa) * density / beta;
}

cudaError_t launch_inject(amps_gpu_ctx* c, const StepArgs& a) {
  InjArgs g{};
  g.nsrc = (int)std::min<size_t>(c->inj.size(), kMaxInj);
  const int nbk[3] = {c->cfg.nbx, c->cfg.nby, c->cfg.nbz};
  int first = 0;
  for (int s = 0; s < g.nsrc; s++) {
    const amps_gpu_ctx::InjSource& S = c->inj[(size_t)s];
    InjDev& D = g.src[s];
    const int ax = S.face >> 1, ta = (ax + 1) % 3, tb = (ax + 2) % 3;
    D.face = S.face;
    D.spec = S.spec;
    // face cells (uniform) or finest-lattice face patches (AMR)
    D.ncell = c->amr ? c->amrdev.nfine[ta] * c->amrdev.nfine[tb] : 64 * nbk[ta] * nbk[tb];
    D.first = first;
    first += D.ncell;
    D.beta = 1.0 / (std::sqrt(2.0) * S.vth);
    for (int d = 0; d < 3; d++) D.drift[d] = S.drift[d];
    double n[3] = {0.0, 0.0, 0.0};
    n[ax] = (S.face & 1) ? 1.0 : -1.0;
    D.rate = maxwellian_flux(S.density, S.drift, D.beta, n) / c->cfg.weight[S.spec];
  }
  g.nthreads = first;
  g.dt = c->cfg.dt;
  for (int d = 0; d < 3; d++) {
    g.dx[d] = c->amr ? c->dxf : c->cfg.dx[d];
    g.nbk[d] = nbk[d];
  }
  g.seed = c->inj_seed;
  g.step = c->d_step;
  {
    TimedLaunch t(c, "inject", 2);
    k_inject<<<(unsigned)((g.nthreads + 127) / 128), 128, 0, c->stream>>>(a, g);
    k_step_bump<<<1, 32, 0, c->stream>>>(c->d_step, c->d_flags);
  }
  return cudaGetLastError();
}

cudaError_t launch_push_step(amps_gpu_ctx* c, bool deposit) {
  set_smem_attrs();
  cudaError_t e;
  if (deposit) {
    e = cudaMemsetAsync(c->d_energy, 0, sizeof(double), c->stream);
    if (e != cudaSuccess) return e;
  }
  StepArgs a = step_args(c);
  const dim3 grid(c->nb, AMPS_NC);
  {
    TimedLaunch t(c, deposit ? "push_deposit" : "push");
    if (c->amr) {
      if (deposit)
        k_push_deposit<true, true><<<grid, kWarps * 32, smem_push(true), c->stream>>>(a);
      else
        k_push_deposit<false, true><<<grid, kWarps * 32, smem_push(false), c->stream>>>(a);
    } else if (c->b_center) {
      if (deposit)
        k_push_deposit<true, false, true><<<grid, kWarps * 32, smem_push(true, true), c->stream>>>(a);
      else
        k_push_deposit<false, false, true><<<grid, kWarps * 32, smem_push(false, true), c->stream>>>(a);
    } else {
      if (deposit)
        k_push_deposit<true, false><<<grid, kWarps * 32, smem_push(true), c->stream>>>(a);
      else
        k_push_deposit<false, false><<<grid, kWarps * 32, smem_push(false), c->stream>>>(a);
    }
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (!c->inj.empty()) {
    if ((e = launch_inject(c, a)) != cudaSuccess) return e;
  }
  {
    // while the autotuner compares the chunk sizes, steps alternate them and
    // events bracket the launch (read after the step's synchronisation)
    const bool tune = c->arr_tune_left > 0;
    const int chunk = tune ? ((c->arr_tune_left & 1) ? 32 : 16) : c->arr_chunk;
    if (tune) {
      c->arr_tune_cur = chunk == 32 ? 1 : 0;
      cudaEventRecord(c->arr_ev[0], c->stream);
    }
    TimedLaunch t(c, "arrivals");
    const size_t sm = smem_arr(chunk);
    const int v = (chunk == 32 ? 1 : 0) | (deposit ? 2 : 0) | (c->b_center ? 4 : 0);
    switch (v) {
      case 0: k_arrivals<false, 16><<<grid, kWarps * 32, sm, c->stream>>>(a); break;
      case 1: k_arrivals<false, 32><<<grid, kWarps * 32, sm, c->stream>>>(a); break;
      case 2: k_arrivals<true, 16><<<grid, kWarps * 32, sm, c->stream>>>(a); break;
      case 3: k_arrivals<true, 32><<<grid, kWarps * 32, sm, c->stream>>>(a); break;
      case 4: k_arrivals<false, 16, true><<<grid, kWarps * 32, sm, c->stream>>>(a); break;
      case 5: k_arrivals<false, 32, true><<<grid, kWarps * 32, sm, c->stream>>>(a); break;
      case 6: k_arrivals<true, 16, true><<<grid, kWarps * 32, sm, c->stream>>>(a); break;
      default: k_arrivals<true, 32, true><<<grid, kWarps * 32, sm, c->stream>>>(a); break;
    }
    if (tune) cudaEventRecord(c->arr_ev[1], c->stream);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (deposit) return launch_assemble(c);
  return cudaSuccess;
}

// Overflow entries into the slots vacated in their cells (k_ovf_place); *left
// receives the number that found their cell full.  With the deposit, the
// uniform mesh's corner moments are assembled again.
cudaError_t particles_place_overflow(amps_gpu_ctx* c, long long n_overflow, bool deposit,
                                     long long* left) {
  cudaError_t e = cudaMemsetAsync(c->d_flags + 7, 0, sizeof(unsigned long long), c->stream);
  if (e != cudaSuccess) return e;
  {
    TimedLaunch t(c, "overflow_place");
    const unsigned grid = (unsigned)((n_overflow + kWarps - 1) / kWarps);
    if (deposit && c->b_center)
      k_ovf_place<true, true><<<grid, kWarps * 32, smem_arr(16), c->stream>>>(step_args(c), n_overflow,
                                                                            c->d_flags + 7);
    else if (deposit)
      k_ovf_place<true><<<grid, kWarps * 32, smem_arr(16), c->stream>>>(step_args(c), n_overflow,
                                                                      c->d_flags + 7);
    else
      k_ovf_place<false><<<grid, kWarps * 32, 0, c->stream>>>(step_args(c), n_overflow,
                                                             c->d_flags + 7);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->h_flags + 7, c->d_flags + 7, sizeof(unsigned long long),
                        cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return e;
  *left = (long long)c->h_flags[7];
  // the step assembled the corner moments before the overflow was deposited
  return deposit ? launch_assemble(c) : cudaSuccess;
}

// Relayout after an overflow that the vacated slots did not absorb: every
// cell's particles are copied from the slotted layout into the other buffer at
// new offsets (its count plus its unplaced overflow entries, plus slack), the
// unplaced entries filed behind them, and the buffers swapped.  The overflow
// list occupies the first n_overflow slots of the other buffer, so the new
// layout starts past it (pad) and those slots become holes.  Nothing is
// gathered or re-sorted, and no deposit is redone: k_ovf_place deposited
// every overflow entry.
cudaError_t particles_relayout(amps_gpu_ctx* c, long long n_overflow) {
  cudaStream_t s = c->stream;
  const long long nc = c->ncor, n = c->np;
  const long long pad = (n_overflow + 127) & ~127LL;
  const long long room = c->slots - pad - n;
  if (room < 0) return cudaErrorMemoryAllocation;
  const int other = c->cur ^ 1;
  cudaError_t e = cudaMemcpyAsync(c->d_count, c->d_cnt, sizeof(int) * nc, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) return e;
  // slack scaled so that pad + sum(cap) <= slots
  const long long worst = n + n / 4 + (long long)AMPS_SLACK_MIN * nc;
  int num = 1, den = 1;
  if (worst - n > room) {
    num = (int)std::max(0LL, room / 1024);
    den = (int)std::max(1LL, (worst - n) / 1024 + 1);
  }
  {
    TimedLaunch t(c, "relayout_aux", 2);
    k_ovf_count<<<grid_for(n_overflow, 256), 256, 0, s>>>(n_overflow, c->d_key, c->d_count);
    k_rb_caps<<<(unsigned)((nc + 1 + 255) / 256), 256, 0, s>>>(nc, c->d_count, c->d_tmp, num, den);
  }
  e = scan_ints(c, c->d_tmp, c->d_rank, nc + 1);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_sp[other] + pad, 0xFF, (size_t)(c->slots - pad), s);
  if (e != cudaSuccess) return e;
  {
    TimedLaunch t(c, "relayout");
    const long long threads = nc * 32;
    k_relayout_cells<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
        nc, c->d_base, c->d_cnt, c->d_rank, pad, pbuf(c, c->cur), pbuf(c, other));
  }
  {
    TimedLaunch t(c, "relayout_aux", 2);
    k_ovf_file<<<grid_for(n_overflow, 256), 256, 0, s>>>(n_overflow, c->d_key, c->d_rank, pad,
                                                         c->d_cnt, pbuf(c, other));
    k_offset_copy<<<(unsigned)((nc + 1 + 255) / 256), 256, 0, s>>>(nc + 1, c->d_rank, pad,
                                                                   c->d_base);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_sp[other], 0xFF, (size_t)pad, s);
  if (e != cudaSuccess) return e;
  c->cur = other;
  return cudaSuccess;
}

// Every particle of the slotted layout (buffer cur) into the list buffer
// (cur^1) with its cell as key, for a pass that moves particles and re-bins
// them with rebuild_from_list.
cudaError_t particles_to_list(amps_gpu_ctx* c) {
  cudaError_t e = cudaMemsetAsync(c->d_flags + 4, 0, sizeof(unsigned long long), c->stream);
  if (e != cudaSuccess) return e;
  TimedLaunch t(c, "gather");
  const long long threads = c->ncor * 32;
  k_gather_valid<<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
      c->ncor, c->d_base, c->d_cnt, pbuf(c, c->cur), pbuf(c, c->cur ^ 1), c->d_key, c->d_flags + 4);
  return cudaGetLastError();
}

// Relativistic Boris move of every particle: compact layout -> list buffer,
// sub-stepped move with new keys, counting-sort rebuild.  Sub-step total in
// flags[4] (read back by the caller).
cudaError_t launch_relboris(amps_gpu_ctx* c, const double* E, const double* B, double dt_total,
                            double c_light, long long max_sub, bool rel) {
  cudaError_t e = cudaMemsetAsync(c->d_flags + 4, 0, 2 * sizeof(unsigned long long), c->stream);
  if (e != cudaSuccess) return e;
  {
    TimedLaunch t(c, "relboris_gather");
    const long long threads = c->ncor * 32;
    k_gather_valid<<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
        c->ncor, c->d_base, c->d_cnt, pbuf(c, c->cur), pbuf(c, c->cur ^ 1), c->d_key,
        c->d_flags + 4);
  }
  if (c->amr) {
    AmrRelBorisArgs a;
    a.d = pbuf(c, c->cur ^ 1);
    a.key = c->d_key;
    a.n = c->np;
    a.m = c->amrdev;
    a.ctab = c->d_ctab;
    a.hs = c->d_hs;
    a.hp = c->d_hp;
    a.hw = c->d_hw;
    a.nvc = c->nvc;
    a.E = E;
    a.B = B;
    for (int d = 0; d < 3; d++) a.x0[d] = c->cfg.x0[d];
    a.dxf = c->dxf;
    for (int sp = 0; sp < AMPS_GPU_MAX_SPECIES; sp++) {
      a.qm[sp] = sp < c->cfg.nspec ? c->cfg.charge[sp] / c->cfg.mass[sp] : 0.0;
      a.qabs_over_m[sp] = sp < c->cfg.nspec ? fabs(c->cfg.charge[sp]) / c->cfg.mass[sp] : 0.0;
    }
    a.dt_total = dt_total;
    a.c_light = c_light;
    a.max_sub = max_sub;
    a.flags = c->d_flags;
    a.nsub = c->d_flags + 5;
    a.open = c->open_axes;
    {
      TimedLaunch t(c, rel ? "relboris" : "boris");
      if (rel)
        k_amr_relboris<true><<<grid_for(c->np, 256), 256, 0, c->stream>>>(a);
      else
        k_amr_relboris<false><<<grid_for(c->np, 256), 256, 0, c->stream>>>(a);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return rebuild_from_list(c, c->np);
  }
  RelBorisArgs a;
  a.d = pbuf(c, c->cur ^ 1);
  a.key = c->d_key;
  a.n = c->np;
  a.nbr = c->d_nbr;
  a.ncor = c->ncor;
  a.E = E;
  a.B = B;
  a.nbk[0] = c->cfg.nbx; a.nbk[1] = c->cfg.nby; a.nbk[2] = c->cfg.nbz;
  for (int d = 0; d < 3; d++) { a.x0[d] = c->cfg.x0[d]; a.dx[d] = c->cfg.dx[d]; }
  for (int sp = 0; sp < AMPS_GPU_MAX_SPECIES; sp++) {
    a.qm[sp] = sp < c->cfg.nspec ? c->cfg.charge[sp] / c->cfg.mass[sp] : 0.0;
    a.qabs_over_m[sp] = sp < c->cfg.nspec ? fabs(c->cfg.charge[sp]) / c->cfg.mass[sp] : 0.0;
  }
  a.dt_total = dt_total;
  a.c_light = c_light;
  a.max_sub = max_sub;
  a.flags = c->d_flags;
  a.nsub = c->d_flags + 5;
  a.open = c->open_axes;
  {
    TimedLaunch t(c, rel ? "relboris" : "boris");
    if (rel)
      k_relboris<true><<<grid_for(c->np, 256), 256, 0, c->stream>>>(a);
    else
      k_relboris<false><<<grid_for(c->np, 256), 256, 0, c->stream>>>(a);
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return rebuild_from_list(c, c->np);
}

cudaError_t launch_import_fp64(amps_gpu_ctx* c, const double* d_x, const double* d_v,
                               const uint8_t* d_spec_in, const double* d_wc, long long n) {
  if (c->amr) {
    ImportAmrArgs a;
    a.x = d_x; a.v = d_v; a.sp = d_spec_in; a.wc = d_wc;
    a.d = pbuf(c, c->cur ^ 1);
    a.key = c->d_key;
    a.flags = c->d_flags;
    a.n = n;
    a.m = c->amrdev;
    for (int d = 0; d < 3; d++) a.x0[d] = c->cfg.x0[d];
    a.dxf = c->dxf;
    a.nspec = c->cfg.nspec;
    {
      TimedLaunch t(c, "import");
      k_import_amr<<<grid_for(n, 256), 256, 0, c->stream>>>(a);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    c->np = n;
    set_next_id(c, n);
    return rebuild_from_list(c, n);
  }
  ImportArgs a;
  a.x = d_x; a.v = d_v; a.sp = d_spec_in; a.wc = d_wc;
  a.d = pbuf(c, c->cur ^ 1);
  a.key = c->d_key;
  a.flags = c->d_flags;
  a.n = n;
  a.nbk[0] = c->cfg.nbx; a.nbk[1] = c->cfg.nby; a.nbk[2] = c->cfg.nbz;
  for (int d = 0; d < 3; d++) { a.x0[d] = c->cfg.x0[d]; a.dx[d] = c->cfg.dx[d]; }
  a.nspec = c->cfg.nspec;
  {
    TimedLaunch t(c, "import");
    k_import<<<grid_for(n, 256), 256, 0, c->stream>>>(a);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  c->np = n;
  set_next_id(c, n);
  return rebuild_from_list(c, n);
}

cudaError_t launch_import_local(amps_gpu_ctx* c, const float* d_u, const float* d_v,
                                const uint8_t* d_sp, const int32_t* d_block, const float* d_wc,
                                long long n) {
  {
    TimedLaunch t(c, "import");
    k_import_local<<<grid_for(n, 256), 256, 0, c->stream>>>(n, d_u, d_v, d_sp, d_block, d_wc,
                                                             c->nb, c->cfg.nspec, pbuf(c, c->cur ^ 1),
                                                             c->d_key, c->d_flags);
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  c->np = n;
  set_next_id(c, n);
  return rebuild_from_list(c, n);
}

cudaError_t launch_export(amps_gpu_ctx* c, double* d_x, double* d_v, uint8_t* d_sp,
                          int32_t* d_blk, int32_t* d_cel, uint32_t* d_id) {
  cudaError_t e = cudaMemcpyAsync(c->d_tmp, c->d_cnt, sizeof(int) * c->ncor,
                                  cudaMemcpyDeviceToDevice, c->stream);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(c->d_tmp + c->ncor, 0, sizeof(int), c->stream);
  if (e != cudaSuccess) return e;
  e = scan_ints(c, c->d_tmp, c->d_tmp, c->ncor + 1);
  if (e != cudaSuccess) return e;
  TimedLaunch t(c, "export");
  k_export<<<(unsigned)((c->ncor + 255) / 256), 256, 0, c->stream>>>(
      c->ncor, c->d_base, c->d_cnt, c->d_tmp, pbuf(c, c->cur), c->cfg.nbx, c->cfg.nby,
      c->cfg.x0[0], c->cfg.x0[1], c->cfg.x0[2], c->cfg.dx[0], c->cfg.dx[1], c->cfg.dx[2], d_x, d_v,
      d_sp, d_blk, d_cel, d_id, c->amrdev, c->dxf);
  return cudaGetLastError();
}
