// Shared declarations of libamps_gpu.so: device context, launch helpers,
// block-structured index arithmetic.
//
// Data layout in HBM (one context = one periodic mesh of 8^3-cell blocks)
//   blocks own their 512 low corners and 512 cells: corner id = b*512 + i + 8j + 64k
//   FP64 vectors are component-major: v[comp*ncor + corner]
//   mass matrix M: 243 FP32 coefficient planes, M[e*ncor + corner] (coalesced per
//              plane; the deposited values are FP32 sums, widened where FP64 is needed)
//   particles: FP32 SoA (u: block-local offset in cell units, v), species byte,
//              optional 32-bit id; every cell owns a slot range with slack
//   per-block FP32 field stencils (9^3 corners incl. the +1 halo) for the push
//   and deposit kernels, contiguous per block so one bulk TMA copy stages them.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/amps_gpu.h"

#define AMPS_NC 8
#define AMPS_CPB 512        // cells (and owned corners) per block
#define AMPS_SC 729         // stencil corners per block (9^3)
#define AMPS_PUSH_STRIDE 8  // floats per stencil corner for the push: E3 B3 pad2
#define AMPS_DEP_STRIDE 4   // floats per stencil corner for the deposit: B3 pad1
#define AMPS_CSC 1000       // centre stencil per block (10^3 cell centres incl. the +-1 halo)
#define AMPS_SLACK_MIN 32   // slack slots per cell on top of count/4 (rebuild)
#define AMPS_CELLM 243      // per-cell mass-matrix partials: 27 weight monomials x 9

struct KernelTimer {
  const char* name;
  double ms = 0.0;
  long long launches = 0;
};

// Device view of a block-structured AMR mesh for the particle kernels (null
// pointers on uniform meshes).  Block origins are integers on the finest
// lattice and cell sizes powers of two of the finest one, so a particle's
// block-local FP32 offset converts between blocks with one rounding.
struct AmrDev {
  int nfine[3];            // finest cells per axis
  const int* fine_map;     // finest block -> leaf block
  const int* borg;         // nb*3 origins, finest-cell units
  const int* bscale;       // nb: finest cells per cell (2^(lmax-level))
  const float* bdtdx;      // nb: dt / dx
  const float* binvvol;    // nb: 1 / dx^3
};

struct PrecondState;

struct amps_gpu_ctx {
  amps_gpu_config cfg;
  int nb = 0;               // blocks
  long long ncor = 0;       // cells (= owned corners on a uniform mesh)
  long long nvc = 0;        // corners carrying unknowns (= ncor uniform, unique corners on AMR)
  cudaStream_t stream = nullptr;
  // device-to-host copies that overlap the producing kernels (created on
  // first use) and the events that order them, one per chunk
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copy_ev[17] = {nullptr};
  std::string err;

  // mesh
  int* d_nbr = nullptr;     // [nb*27] neighbour block, slot (di+1)+3(dj+1)+9(dk+1) (uniform)
  bool amr = false;
  AmrDev amrdev{};          // particle-kernel view (AMR)
  int lmax = 0;
  double dxf = 0.0;         // finest cell size (AMR)
  int* d_ctab = nullptr;    // [nb*729] block-local corner -> unique corner (AMR)
  int* d_hs = nullptr;      // [nvc+1] hanging CSR start (AMR)
  int* d_hp = nullptr;      // hanging parents
  double* d_hw = nullptr;   // hanging weights
  float* d_hwh = nullptr;   // the hanging weights as FP32 pairs (hi, lo)
  float* d_hwl = nullptr;
  // field boundary rows of AMR meshes with open axes (null: fully periodic)
  int* d_bflag = nullptr;   // nvc: 1 on a boundary constraint row
  int* d_bs = nullptr;      // nvc+1 CSR of the donor lists
  int* d_bc = nullptr;
  double* d_bw = nullptr;
  float* d_bwh = nullptr;
  float* d_bwl = nullptr;
  int mesh_open = 0;        // bit d: axis d of the AMR mesh is not periodic
  int neumann = 0;          // bit 2d + high: a Neumann open face (else Dirichlet)
  int* d_fine_map = nullptr;
  int* d_borg = nullptr;      // nb*3 origins, finest-cell units
  int* d_bscale = nullptr;    // nb finest cells per cell
  double* d_bdx = nullptr;    // nb cell sizes
  float* d_bdtdx = nullptr;   // dt/dx per block
  float* d_binvvol = nullptr; // 1/dx^3 per block
  int* d_ss = nullptr;        // identity part of the AMR operator, CSR rows (nvc+1)
  int* d_sc = nullptr;        //   columns
  double* d_sv = nullptr;     //   values
  float* d_svh = nullptr;     //   values as FP32 pairs
  float* d_svl = nullptr;

  // fields (FP64, component-major)
  double* d_En = nullptr;
  double* d_Eh = nullptr;
  double* d_Bc = nullptr;       // centre B^n (current)
  double* d_Bc2 = nullptr;      // scratch for B^{n+1}
  double* d_Bcor_prev = nullptr;
  double* d_Bcor_cur = nullptr;
  double* d_J = nullptr;        // 3*ncor
  float* d_M = nullptr;         // 243*ncor (uniform meshes)
  bool have_moments = false;

  // GMRES workspace
  double* d_rhs = nullptr;
  double* d_x = nullptr;
  double* d_V = nullptr;        // (restart+1) * n
  double* d_w = nullptr;
  double* d_dinv = nullptr;
  double* d_Z = nullptr;        // (restart+1) * n preconditioned directions (learned)
  float* d_dff = nullptr;       // 2n: the Jacobi scaling as FP32 pairs (hi n, lo n)
  double* d_tmpv = nullptr;     // 2n doubles: FP64 copies of Krylov vectors for the
                                // learned network, its sample harvest and the FP64 inner operator
  float* d_y32 = nullptr;       // 3*nvc FP32 accumulation of the inner AMR operator
  bool inner_fp32 = true;       // GMRES inner operator in FP32 (iterative refinement)
  PrecondState* pn = nullptr;   // learned preconditioner (precond.cu)
  // the network's view of the mesh: per block the 10^3 corner region (block
  // corners -1..8) as entries of pc_input(), the 8^3 corners it writes as
  // indices into the corner vectors (-1: not written by this block), the
  // weight set of the block (its refinement level; null on a uniform mesh) and
  // the corners no block writes (z = D v there).  Two variants of the output
  // maps: [0] the network on every block, [1] Jacobi on the blocks whose region
  // reaches a refinement interface (a hanging or missing corner).
  int* d_pc_in = nullptr;       // [nb*1000]
  int* d_pc_out = nullptr;      // active variant [nb*512]
  int* d_pc_set = nullptr;      // [nb]
  int* d_pc_jac = nullptr;      // active variant [pc_njac]
  long long pc_njac = 0;
  int* d_pc_out_v[2] = {nullptr, nullptr};
  int* d_pc_jac_v[2] = {nullptr, nullptr};
  long long pc_njac_v[2] = {0, 0};
  int pc_nsets = 1;
  int pc_iface_blocks = 0;      // blocks that reach a refinement interface
  bool pc_iface_jacobi = false; // variant [1] active
  std::vector<int> h_pc_set;    // [nb]
  std::vector<char> h_pc_iface; // [nb] block reaches a refinement interface

  // launch parameters chosen by the autotuner (field.cu: field_autotune)
  int tune_tb = 256;            // threads per CTA of the operator kernels
  int tune_red = 304;           // maximum CTAs of the reduction sweeps
  int tune_ept = 4;             // minimum elements per thread of the sweeps

  // CUDA graphs of the particle step (capi.cu), keyed by the pointers they bake in
  bool use_graphs = false;
  struct StepGraph {
    bool deposit;
    const void* key[7];
    cudaGraphExec_t exec;
  };
  std::vector<StepGraph> graphs;
  // the first GMRES cycle of a solve as a graph (gmres_solve), keyed by the
  // preconditioner, the Arnoldi steps and the launch shapes it was captured with
  struct SolveGraph {
    int precond, steps, tb, red, ept;
    cudaGraphExec_t exec;
  };
  std::vector<SolveGraph> solve_graphs;
  bool solve_graphs_off = false;  // a capture failed: solves stay eager
  // div E correction (dive.cu): per cell rho_new, rho_old, div E, phi, then the
  // CG vectors f, r, p, Ap and the species-0 corner charge (9 x ncor doubles)
  double* d_dive = nullptr;
  bool dive_have_rho = false;
  // arrivals staged 16 or 32 at a time (k_arrivals<DEP, CHUNK>); the autotuner
  // alternates them over arr_tune_left steps, timed by arr_ev, then keeps the
  // faster (arr_tune_ms: summed ms per variant, arr_tune_n: steps)
  // magnetic field the particles see: false corners (the corner B slots),
  // true cell centres (_PIC_FIELD_SOLVER_B_CENTER_BASED_: centre B^n for the
  // push, B^{n+1} for the deposit, uniform meshes), staged per block as 10^3
  // float4 (B3 pad) in d_stencil_cprev / d_stencil_ccur
  bool b_center = false;
  float* d_stencil_cprev = nullptr;
  float* d_stencil_ccur = nullptr;
  int arr_chunk = 16;
  int arr_tune_left = 0;
  int arr_tune_cur = -1;  // variant of the step in flight, -1: none
  double arr_tune_ms[2] = {0.0, 0.0};
  int arr_tune_n[2] = {0, 0};
  cudaEvent_t arr_ev[2] = {nullptr, nullptr};
  double* d_red = nullptr;      // partial reductions
  double* d_arn = nullptr;      // per-CTA partial sums of the cooperative Arnoldi step
  float* d_xs = nullptr;        // FP32 pair split (hi, lo) of an operator input, 2 x 3*nvc
  double* h_red = nullptr;      // pinned
  int restart = 30;
  int gm_guess[3] = {0, 0, 0};  // per preconditioner: Arnoldi steps of the last first cycle
                                // (steps queued before the host first waits)

  // per-block FP32 stencils
  float* d_stencil_push = nullptr;  // nb * 729 * 8
  float* d_stencil_dep = nullptr;   // nb * 729 * 4

  // particles: two FP32 SoA buffers of `slots` entries.  Buffer `cur` holds the
  // slotted cell layout (cell c owns [base[c], base[c+1]), occupancy cnt[c]);
  // the other one is the unsorted list used by import and overflow recovery.
  long long cap = 0, np = 0, slots = 0;
  float* d_u[2][3] = {{nullptr}};
  float* d_v[2][3] = {{nullptr}};
  uint8_t* d_sp[2] = {nullptr, nullptr};
  float* d_wc[2] = {nullptr, nullptr};  // optional weight correction
  uint32_t* d_id[2] = {nullptr, nullptr};
  int cur = 0;
  bool has_wcorr = false;
  int open_axes = 0;            // bit d: particles leaving through a face of axis d are deleted
  long long deleted_total = 0;  // particles deleted at open faces since creation
  // injection through open faces (particles.cu: k_inject)
  struct InjSource {
    int face, spec;
    double density, drift[3], vth;
  };
  std::vector<InjSource> inj;
  unsigned long long inj_seed = 1;
  unsigned long long* d_step = nullptr;  // device step counter of the injection random streams
  long long injected_total = 0;
  uint32_t next_id = 0;         // id of the next injected particle (import ids are 0..n-1)
  int32_t* d_base = nullptr;    // ncor+1 slot offsets
  int32_t* d_cnt = nullptr;     // ncor occupancy
  int32_t* d_arr = nullptr;     // ncor arrivals in the current step
  int32_t* d_stay = nullptr;    // ncor stayers in the current step
  int32_t* d_tmp = nullptr;     // ncor+1 scratch for scans
  int32_t* d_key = nullptr;     // slots: list keys (import / overflow)
  int32_t* d_rank = nullptr;    // slots: rank inside the destination cell (rebuild)
  int32_t* d_count = nullptr;   // ncor+1 histogram (rebuild)
  int32_t* d_scan_part = nullptr;
  // [0] moved > 1 block, [1] near a cell face, [2] device error, [3] overflow, [4] list tail,
  // [5] deleted at open faces, [6] injected
  unsigned long long* d_flags = nullptr;
  unsigned long long* h_flags = nullptr;  // pinned

  // deposition scratch: per-cell partial sums
  float* d_cellM = nullptr;     // ncor * AMPS_CELLM
  float* d_cellJ = nullptr;     // ncor * 24
  double* d_energy = nullptr;   // [0] particle, [1] wave, [4 + s] max CFL of species s
  double* h_energy = nullptr;   // pinned

  // species moments on corners (species.cu), when sampling is on
  bool spec_on = false;
  float* d_cellS = nullptr;     // [ncor][nspec][10][8] per-cell partials
  double* d_specC = nullptr;    // [10*nspec][nvc] corner values
  float* d_bivh = nullptr;      // AMR: 1/dx^3 per block as an FP32 pair (hi nb, lo nb)
  double* d_amrJ = nullptr;     // AMR corner-layout moments (export_moments)
  double* d_amrM = nullptr;
  int* d_spec_start = nullptr;  // corner -> (cell*8 + corner-of-cell) CSR
  int* d_spec_ent = nullptr;

  // device staging of host <-> device layout conversions (layout.cu)
  double* d_hstage = nullptr;
  size_t hstage_bytes = 0;

  // timing
  bool timing = false;
  std::vector<KernelTimer> timers;
  std::vector<cudaEvent_t> ev_pool;
};

// ---- error helpers ----
amps_gpu_status set_err(amps_gpu_ctx* c, amps_gpu_status s, const std::string& msg);
amps_gpu_status cuda_check(amps_gpu_ctx* c, cudaError_t e, const char* what);

// Brackets a launch with CUDA events on the context stream when timing is on.
struct TimedLaunch {
  amps_gpu_ctx* c;
  int slot;
  cudaEvent_t a = nullptr, b = nullptr;
  int nk = 1;
  TimedLaunch(amps_gpu_ctx* ctx, const char* name, int kernels = 1);
  ~TimedLaunch();
};
void flush_timers(amps_gpu_ctx* c);

// ---- kernel launchers (particles.cu) ----
cudaError_t launch_pack_stencils(amps_gpu_ctx* c, const double* Eh, const double* Bprev,
                                 const double* Bcur);
cudaError_t launch_push_step(amps_gpu_ctx* c, bool deposit);
void particles_prepare();

// ---- host <-> device layout conversion (layout.cu) ----
amps_gpu_status layout_upload(amps_gpu_ctx* c, const double* host, void* dev, long long n,
                              int ncomp, bool dev_f32);
amps_gpu_status layout_download(amps_gpu_ctx* c, const void* dev, double* host, long long n,
                                int ncomp, bool dev_f32);
amps_gpu_status layout_cell_moments(amps_gpu_ctx* c, double* hJ, double* hM);
// device address of a page-locked host array (kernels write it across the host
// link directly), or null for pageable memory
double* host_mapped(double* host);
cudaError_t launch_relboris(amps_gpu_ctx* c, const double* E, const double* B, double dt_total,
                            double c_light, long long max_sub, bool rel = true);
cudaError_t launch_deposit(amps_gpu_ctx* c);
void set_next_id(amps_gpu_ctx* c, long long n);
// counting sort of the list buffer into the slotted layout (keys in d_key)
cudaError_t rebuild_from_list(amps_gpu_ctx* c, long long n);
// its placement half: d_count, d_key and d_rank already filled
cudaError_t place_ranked(amps_gpu_ctx* c, long long n);
// species moments on corners (species.cu)
amps_gpu_status species_setup(amps_gpu_ctx* c, bool on);
void species_free(amps_gpu_ctx* c);
amps_gpu_status amr_export_corner_moments(amps_gpu_ctx* c, double* J, double* M);
cudaError_t launch_species_moments(amps_gpu_ctx* c);
cudaError_t particles_place_overflow(amps_gpu_ctx* c, long long n_overflow, bool deposit,
                                     long long* left);
cudaError_t particles_relayout(amps_gpu_ctx* c, long long n_overflow);
cudaError_t particles_to_list(amps_gpu_ctx* c);
cudaError_t launch_import_fp64(amps_gpu_ctx* c, const double* d_x, const double* d_v,
                               const uint8_t* d_spec_in, const double* d_wc, long long n);
cudaError_t launch_import_local(amps_gpu_ctx* c, const float* d_u, const float* d_v,
                                const uint8_t* d_sp, const int32_t* d_block, const float* d_wc,
                                long long n);
cudaError_t launch_export(amps_gpu_ctx* c, double* d_x, double* d_v, uint8_t* d_sp,
                          int32_t* d_blk, int32_t* d_cel, uint32_t* d_id);

// ---- field launchers (field.cu) ----
cudaError_t launch_rhs(amps_gpu_ctx* c);
cudaError_t launch_matvec(amps_gpu_ctx* c, const double* x, const double* dinv, double* y);
// the same operator evaluated in FP32 arithmetic (inner GMRES iterations)
cudaError_t launch_matvec32(amps_gpu_ctx* c, const double* x, const double* dinv, double* y);
// Input of the inner operator on a Krylov vector: v as FP32 pairs (vh, vl) or,
// for the flexible directions, as doubles (vd); the scaling D as FP32 pairs
// (dh, dl) or none.  The operator computes w = A (D v) and writes it as FP32
// pairs; FP32 pair vectors of length n hold hi in [0, n) and lo in [n, 2n) of
// the same bytes a double vector of length n would take.
struct OpIn {
  const double* vd;
  const float* vh;
  const float* vl;
  const float* dh;
  const float* dl;
  bool xf_ready;  // fp32(D v) already in the context's scratch (written by the Arnoldi step)
};
cudaError_t launch_matvec32_ff(amps_gpu_ctx* c, const OpIn& in, float* wh, float* wl);
// xf = fp32(D v), the FP32 operator's input
cudaError_t launch_in_f32(amps_gpu_ctx* c, const OpIn& in, float* xf);
cudaError_t launch_amr_matvec32_ff(amps_gpu_ctx* c, const OpIn& in, float* wh, float* wl);
cudaError_t launch_jacobi_diag(amps_gpu_ctx* c);
cudaError_t launch_update_b(amps_gpu_ctx* c);
cudaError_t launch_c2n(amps_gpu_ctx* c, const double* Bcen, double* Bcor);
cudaError_t launch_update_e(amps_gpu_ctx* c);
amps_gpu_status gmres_solve(amps_gpu_ctx* c, double tol, int maxit, int precond,
                            amps_gpu_solve_stats* st);
// times candidate launch shapes of the operator and reduction kernels on the
// context's own data and keeps the fastest; ms[6] receives the timings
amps_gpu_status field_autotune(amps_gpu_ctx* c, double* ms);

// ---- AMR field launchers (amr_field.cu); the launchers above dispatch to
//      them when the context holds an AMR mesh ----
cudaError_t launch_amr_pack(amps_gpu_ctx* c, const double* Eh, const double* Bprev,
                            const double* Bcur);
cudaError_t launch_amr_matvec(amps_gpu_ctx* c, const double* x, const double* dinv, double* y);
cudaError_t launch_amr_matvec32(amps_gpu_ctx* c, const double* x, const double* dinv, double* y);
cudaError_t launch_amr_rhs(amps_gpu_ctx* c);
cudaError_t launch_amr_jacobi(amps_gpu_ctx* c);
cudaError_t launch_amr_update_b(amps_gpu_ctx* c);
cudaError_t launch_amr_c2n(amps_gpu_ctx* c, const double* Bcen, double* Bcor);
cudaError_t launch_amr_update_e(amps_gpu_ctx* c);
cudaError_t launch_amr_fix_hanging(amps_gpu_ctx* c, double* F);

// ---- device helpers ----
__host__ __device__ inline int nbr_slot(int ox, int oy, int oz) {
  return (ox + 1) + 3 * (oy + 1) + 9 * (oz + 1);
}

// FP64-accurate sums of products at FP32 throughput (GB300 issues FP32 FMAs at
// 64x its FP64 rate): x = xh + xl split into FP32 (xh = fp32(x)); a product
// with an FP32 coefficient m is m xh exactly (its rounding error recovered by
// an FMA) plus m xl.  The leading parts are summed with an error-free TwoSum
// per step (Knuth), whose exact errors go with the small parts into a second
// FP32 sum (the cascaded summation of Ogita, Rump and Oishi); the two are
// combined in FP64.  Error ~1e-14 of the sum of |terms| for 81 terms.  The
// arithmetic uses the _rn intrinsics, which the compiler never contracts into
// FMAs (a contraction would break the error-free transformations).
struct FF {
  float s, q;
};
__device__ __forceinline__ void ff_acc(FF& a, float ph, float pl) {
  const float t = __fadd_rn(a.s, ph);
  const float bp = __fsub_rn(t, a.s);
  const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(ph, bp));
  a.s = t;
  a.q = __fadd_rn(a.q, __fadd_rn(err, pl));
}
// a += m (xh + xl), m exact in FP32
__device__ __forceinline__ void ff_add(FF& a, float m, float xh, float xl) {
  const float ph = __fmul_rn(m, xh);
  ff_acc(a, ph, fmaf(m, xl, fmaf(m, xh, -ph)));
}
// a += (kh + kl)(xh + xl), an FP64 coefficient split into FP32 pairs
__device__ __forceinline__ void ff_add2(FF& a, float kh, float kl, float xh, float xl) {
  const float ph = __fmul_rn(kh, xh);
  ff_acc(a, ph, fmaf(kh, xl, fmaf(kl, xh, fmaf(kh, xh, -ph))));
}
__device__ __forceinline__ double ff_value(const FF& a) { return (double)a.s + (double)a.q; }
// (s, q) renormalised so that q is below half an ulp of s (fast two-sum)
__device__ __forceinline__ FF ff_norm(const FF& a) {
  const float t = __fadd_rn(a.s, a.q);
  return FF{t, __fsub_rn(a.q, __fsub_rn(t, a.s))};
}
// (xh + xl)(kh + kl) as a pair
__device__ __forceinline__ FF ff_mul(float xh, float xl, float kh, float kl) {
  const float ph = __fmul_rn(xh, kh);
  return FF{ph, fmaf(xh, kl, fmaf(xl, kh, fmaf(xh, kh, -ph)))};
}
// D v as a pair at element t (FP64 input split, FP32 pair input scaled in pairs)
__device__ __forceinline__ FF opin_value(const OpIn& in, long long t) {
  if (in.vd) {
    const double v = in.vd[t];
    const float h = (float)v;
    return FF{h, (float)(v - (double)h)};
  }
  if (!in.dh) return FF{in.vh[t], in.vl[t]};
  return ff_mul(in.vh[t], in.vl[t], in.dh[t], in.dl[t]);
}

// Input of the learned preconditioner at one entry e of its region map: D v at
// a free corner (e >= 0), nothing (e == -1: no corner of the block's lattice
// there), or at a hanging corner h (e = -2 - h) D v interpolated from its
// parents (hs/hp/hw: the hanging-corner CSR of the mesh).
__device__ __forceinline__ double pc_input(int e, int ch, long long nvc, const double* __restrict__ v,
                                           const double* __restrict__ dinv, const int* __restrict__ hs,
                                           const int* __restrict__ hp, const double* __restrict__ hw) {
  if (e >= 0) return dinv[ch * nvc + e] * v[ch * nvc + e];
  if (e == -1) return 0.0;
  const int h = -2 - e;
  double s = 0.0;
  for (int q = hs[h]; q < hs[h + 1]; q++) {
    const long long p = hp[q];
    s += hw[q] * dinv[ch * nvc + p] * v[ch * nvc + p];
  }
  return s;
}

// Corner (or cell) id of block-local index (i,j,k) in [-8,16): follows the
// neighbour table for indices outside [0,8).
__device__ __forceinline__ int local_id(const int* __restrict__ nbr, int b, int i, int j, int k) {
  int ox = (i < 0) ? -1 : ((i >= AMPS_NC) ? 1 : 0);
  int oy = (j < 0) ? -1 : ((j >= AMPS_NC) ? 1 : 0);
  int oz = (k < 0) ? -1 : ((k >= AMPS_NC) ? 1 : 0);
  int bb = (ox | oy | oz) ? __ldg(nbr + b * 27 + nbr_slot(ox, oy, oz)) : b;
  return bb * AMPS_CPB + (i - AMPS_NC * ox) + AMPS_NC * ((j - AMPS_NC * oy) + AMPS_NC * (k - AMPS_NC * oz));
}

// FP32 -> FP64 widening with integer operations (exact for zero and normal
// numbers; GB300's FP64 pipe is narrow, the integer pipe is not).
__device__ __forceinline__ double widen(float f) {
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xFFu;
  if (e == 0u || e == 0xFFu) return (double)f;  // zero, subnormal, inf, nan
  const unsigned long long d = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)(e + 896u) << 52) |
                               ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)d);
}

// 27-slot index of offset (di,dj,dk): digits {0,-1,+1} -> {0,1,2}
__host__ __device__ inline int mm_slot(int di, int dj, int dk) {
  auto dig = [](int o) { return o == 0 ? 0 : (o < 0 ? 1 : 2); };
  return dig(di) + 3 * dig(dj) + 9 * dig(dk);
}
