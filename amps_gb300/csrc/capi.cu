// C ABI of libamps_gpu.so: context lifetime, host<->device transfers, and the
// step sequencing of PIC::TimeStep's ECSIM track (src/pic/pic_time_step.cpp:403-551).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <unordered_map>

#include "amr_mesh.h"
#include "common.cuh"
#include "precond.cuh"

cudaError_t launch_add(amps_gpu_ctx* c, const double* a, const double* b, double* o, long long n);

// ---------------------------------------------------------------------------
amps_gpu_status set_err(amps_gpu_ctx* c, amps_gpu_status s, const std::string& msg) {
  if (c) c->err = msg;
  return s;
}

amps_gpu_status cuda_check(amps_gpu_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return AMPS_GPU_OK;
  return set_err(c, AMPS_GPU_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

struct Pending {
  int slot;
  cudaEvent_t a, b;
  int nk;
};
// pending timed launches per context
std::vector<Pending>& pending(amps_gpu_ctx* c) {
  static std::vector<std::pair<amps_gpu_ctx*, std::vector<Pending>>> tab;
  for (auto& e : tab)
    if (e.first == c) return e.second;
  tab.emplace_back(c, std::vector<Pending>());
  return tab.back().second;
}

cudaEvent_t take_event(amps_gpu_ctx* c) {
  if (!c->ev_pool.empty()) {
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

}  // namespace

TimedLaunch::TimedLaunch(amps_gpu_ctx* ctx, const char* name, int kernels)
    : c(ctx), slot(-1), nk(kernels) {
  if (!c->timing) return;
  for (size_t i = 0; i < c->timers.size(); i++)
    if (std::strcmp(c->timers[i].name, name) == 0) slot = (int)i;
  if (slot < 0) {
    KernelTimer t;
    t.name = name;
    c->timers.push_back(t);
    slot = (int)c->timers.size() - 1;
  }
  a = take_event(c);
  b = take_event(c);
  cudaEventRecord(a, c->stream);
}

TimedLaunch::~TimedLaunch() {
  if (slot < 0) return;
  cudaEventRecord(b, c->stream);
  pending(c).push_back(Pending{slot, a, b, nk});
}

void flush_timers(amps_gpu_ctx* c) {
  auto& pv = pending(c);
  if (pv.empty()) return;
  cudaStreamSynchronize(c->stream);
  for (auto& p : pv) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    c->timers[p.slot].ms += ms;
    c->timers[p.slot].launches += p.nk;
    c->ev_pool.push_back(p.a);
    c->ev_pool.push_back(p.b);
  }
  pv.clear();
}

namespace {

template <class T>
cudaError_t dalloc(T** p, size_t count) {
  return cudaMalloc(reinterpret_cast<void**>(p), std::max<size_t>(count, 1) * sizeof(T));
}

// fields: host layout (interleaved) <-> device layout (component-major), on the GPU
amps_gpu_status upload_vec3(amps_gpu_ctx* c, const double* host, double* dev, long long n) {
  return layout_upload(c, host, dev, n, 3, false);
}

amps_gpu_status download_vec3(amps_gpu_ctx* c, const double* dev, double* host, long long n) {
  return layout_download(c, dev, host, n, 3, false);
}

// staging buffers for particle import/export (allocated on first use)
struct Staging {
  double* x = nullptr;   // 3n doubles (also 3n floats for the local import)
  double* v = nullptr;
  double* wc = nullptr;
  uint8_t* sp = nullptr;
  int32_t* i0 = nullptr;
  int32_t* i1 = nullptr;
  uint32_t* id = nullptr;
  long long cap = 0;
  void release() {
    cudaFree(x); cudaFree(v); cudaFree(wc); cudaFree(sp); cudaFree(i0); cudaFree(i1); cudaFree(id);
    x = v = wc = nullptr; sp = nullptr; i0 = i1 = nullptr; id = nullptr;
    cap = 0;
  }
};
std::vector<std::pair<amps_gpu_ctx*, Staging>>& staging_tab() {
  static std::vector<std::pair<amps_gpu_ctx*, Staging>> t;
  return t;
}
Staging* staging(amps_gpu_ctx* c, long long need) {
  auto& t = staging_tab();
  Staging* s = nullptr;
  for (auto& e : t)
    if (e.first == c) s = &e.second;
  if (!s) {
    t.emplace_back(c, Staging());
    s = &t.back().second;
  }
  if (s->cap < need) {
    s->release();
    if (dalloc(&s->x, 3 * need) || dalloc(&s->v, 3 * need) || dalloc(&s->wc, need) ||
        dalloc(&s->sp, need) || dalloc(&s->i0, need) || dalloc(&s->i1, need) ||
        dalloc(&s->id, need)) {
      s->release();
      return nullptr;
    }
    s->cap = need;
  }
  return s;
}
void staging_free(amps_gpu_ctx* c) {
  auto& t = staging_tab();
  for (size_t i = 0; i < t.size(); i++)
    if (t[i].first == c) {
      t[i].second.release();
      t.erase(t.begin() + i);
      return;
    }
}

// Reads the device flags (one synchronisation).  Overflow is returned, not an error.
amps_gpu_status check_flags(amps_gpu_ctx* c, long long* out_of_block, long long* ulp,
                            long long* overflow) {
  amps_gpu_status s = cuda_check(
      c, cudaMemcpyAsync(c->h_flags, c->d_flags, 4 * sizeof(unsigned long long),
                         cudaMemcpyDeviceToHost, c->stream),
      "read flags");
  if (s) return s;
  s = cuda_check(c, cudaStreamSynchronize(c->stream), "synchronize");
  if (s) return s;
  if (out_of_block) *out_of_block = (long long)c->h_flags[0];
  if (ulp) *ulp = (long long)c->h_flags[1];
  if (overflow) *overflow = (long long)c->h_flags[3];
  if (c->h_flags[2]) {
    return set_err(c, AMPS_GPU_DEVICE_TIMEOUT,
                   "device reported " + std::to_string(c->h_flags[2]) +
                       " bounded-wait timeouts or invalid particle records");
  }
  return AMPS_GPU_OK;
}

amps_gpu_status reset_flags(amps_gpu_ctx* c) {
  return cuda_check(c, cudaMemsetAsync(c->d_flags, 0, 7 * sizeof(unsigned long long), c->stream),
                    "reset flags");
}

// The launch sequence of one particle step: flag reset, stencil pack, push
// (+ deposit), arrivals (+ assembly), flag read-back.
cudaError_t enqueue_particle_step(amps_gpu_ctx* c, bool deposit) {
  cudaError_t e = cudaMemsetAsync(c->d_flags, 0, 7 * sizeof(unsigned long long), c->stream);
  if (e == cudaSuccess) e = launch_pack_stencils(c, c->d_Eh, c->d_Bcor_prev, c->d_Bcor_cur);
  if (e == cudaSuccess) e = launch_push_step(c, deposit);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->h_flags, c->d_flags, 7 * sizeof(unsigned long long),
                        cudaMemcpyDeviceToHost, c->stream);
  return e;
}

// The same sequence as a CUDA graph, captured once per set of buffers it reads
// (the corner-B slots swap every field solve, so two graphs alternate).
cudaError_t launch_particle_step_graph(amps_gpu_ctx* c, bool deposit) {
  const void* key[7] = {c->d_Eh, c->d_Bcor_prev, c->d_Bcor_cur,
                        (const void*)((uintptr_t)c->d_u[c->cur][0] ^ (c->has_wcorr ? 1u : 0u)),
                        (const void*)(uintptr_t)c->arr_chunk, c->b_center ? c->d_Bc : nullptr,
                        c->b_center ? c->d_Bc2 : nullptr};
  for (auto& g : c->graphs)
    if (g.deposit == deposit && std::memcmp(g.key, key, sizeof(key)) == 0)
      return cudaGraphLaunch(g.exec, c->stream);
  particles_prepare();
  cudaGraph_t graph;
  cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaError_t e1 = enqueue_particle_step(c, deposit);
  e = cudaStreamEndCapture(c->stream, &graph);
  if (e1 != cudaSuccess) return e1;
  if (e != cudaSuccess) return e;
  amps_gpu_ctx::StepGraph g;
  g.deposit = deposit;
  std::memcpy(g.key, key, sizeof(key));
  e = cudaGraphInstantiate(&g.exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return e;
  if (c->graphs.size() >= 8) {
    cudaGraphExecDestroy(c->graphs.front().exec);
    c->graphs.erase(c->graphs.begin());
  }
  c->graphs.push_back(g);
  return cudaGraphLaunch(g.exec, c->stream);
}

// flags already copied to h_flags by the step: interpret them after a sync
amps_gpu_status read_step_flags(amps_gpu_ctx* c, long long* out_of_block, long long* ulp,
                                long long* overflow) {
  amps_gpu_status s = cuda_check(c, cudaStreamSynchronize(c->stream), "synchronize");
  if (s) return s;
  if (out_of_block) *out_of_block = (long long)c->h_flags[0];
  if (ulp) *ulp = (long long)c->h_flags[1];
  if (overflow) *overflow = (long long)c->h_flags[3];
  // particles that left through open faces are gone from the layout, the
  // injected ones are in it
  c->np += (long long)c->h_flags[6] - (long long)c->h_flags[5];
  c->deleted_total += (long long)c->h_flags[5];
  c->injected_total += (long long)c->h_flags[6];
  c->next_id += (uint32_t)c->h_flags[6];
  if (c->h_flags[2])
    return set_err(c, AMPS_GPU_DEVICE_TIMEOUT,
                   "device reported " + std::to_string(c->h_flags[2]) +
                       " bounded-wait timeouts or invalid particle records");
  return AMPS_GPU_OK;
}

// One particle step (push, optionally fused with the deposit), with recovery
// when the slack of some destination cell overflowed.
amps_gpu_status particle_step(amps_gpu_ctx* c, bool deposit, long long* out_of_block,
                              long long* near_face) {
  amps_gpu_status s;
  // the autotuner's arrivals comparison runs on stream launches
  const bool graph = c->use_graphs && !c->timing && c->arr_tune_left == 0;
  c->arr_tune_cur = -1;
  if ((s = cuda_check(c, graph ? launch_particle_step_graph(c, deposit)
                               : enqueue_particle_step(c, deposit),
                      "particle step")))
    return s;
  long long ovf = 0;
  if ((s = read_step_flags(c, out_of_block, near_face, &ovf))) return s;
  if (c->arr_tune_cur >= 0) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->arr_ev[0], c->arr_ev[1]) == cudaSuccess) {
      c->arr_tune_ms[c->arr_tune_cur] += ms;
      c->arr_tune_n[c->arr_tune_cur]++;
    }
    if (--c->arr_tune_left == 0 && c->arr_tune_n[0] > 0 && c->arr_tune_n[1] > 0)
      c->arr_chunk = c->arr_tune_ms[1] / c->arr_tune_n[1] < c->arr_tune_ms[0] / c->arr_tune_n[0] ? 32 : 16;
    c->arr_tune_cur = -1;
  }
  if (ovf > 0) {
    // some cell ran out of slack: the overflowed arrivals are deposited and
    // go to the slots their cells' movers vacated; when a cell is full the
    // layout is rebuilt from itself with new slack
    long long left = 0;
    if ((s = cuda_check(c, particles_place_overflow(c, ovf, deposit, &left), "overflow placement")))
      return s;
    if (left > 0 && (s = cuda_check(c, particles_relayout(c, ovf), "overflow relayout"))) return s;
    if ((s = check_flags(c, nullptr, nullptr, nullptr))) return s;
  }
  if (deposit && (s = cuda_check(c, launch_species_moments(c), "species moments"))) return s;
  return AMPS_GPU_OK;
}

}  // namespace

// ===========================================================================
namespace {

amps_gpu_status check_config(const amps_gpu_config* cfg) {
  if (cfg->nspec <= 0 || cfg->nspec > AMPS_GPU_MAX_SPECIES || cfg->dt <= 0.0 ||
      cfg->theta <= 0.0 || cfg->particle_capacity < 0)
    return AMPS_GPU_INVALID_ARG;
  for (int s = 0; s < cfg->nspec; s++)
    if (cfg->mass[s] <= 0.0) return AMPS_GPU_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return AMPS_GPU_NO_DEVICE;
  if (cfg->device < 0 || cfg->device >= ndev) return AMPS_GPU_INVALID_ARG;
  if (cudaSetDevice(cfg->device) != cudaSuccess) return AMPS_GPU_CUDA_ERROR;
  return AMPS_GPU_OK;
}

// Allocations and initial state shared by uniform and AMR contexts (c->nb,
// c->ncor, c->nvc, c->amr set by the caller).  Corner vectors hold 3*nvc
// doubles, cell vectors 3*ncor; the 243-term corner mass matrix exists on
// uniform meshes only (AMR solves read the per-cell partials).
bool alloc_context(amps_gpu_ctx* c) {
  const long long nc = c->ncor, nv = c->nvc, slots = c->slots;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  bool ok = e == cudaSuccess;
  ok = ok && !dalloc(&c->d_En, 3 * nv) && !dalloc(&c->d_Eh, 3 * nv) && !dalloc(&c->d_Bc, 3 * nc) &&
       !dalloc(&c->d_Bc2, 3 * nc) && !dalloc(&c->d_Bcor_prev, 3 * nv) &&
       !dalloc(&c->d_Bcor_cur, 3 * nv);
  if (!c->amr) ok = ok && !dalloc(&c->d_J, 3 * nc) && !dalloc(&c->d_M, 243 * nc);
  if (c->amr) ok = ok && !dalloc(&c->d_y32, 3 * nv);
  ok = ok && !dalloc(&c->d_rhs, 3 * nv) && !dalloc(&c->d_x, 3 * nv) &&
       !dalloc(&c->d_V, (size_t)(c->restart + 1) * 3 * nv) && !dalloc(&c->d_w, 3 * nv) &&
       !dalloc(&c->d_dinv, 3 * nv) && !dalloc(&c->d_red, 12288);
  ok = ok && cudaMallocHost(&c->h_red, 128 * sizeof(double)) == cudaSuccess;
  ok = ok && !dalloc(&c->d_stencil_push, (size_t)c->nb * AMPS_SC * AMPS_PUSH_STRIDE) &&
       !dalloc(&c->d_stencil_dep, (size_t)c->nb * AMPS_SC * AMPS_DEP_STRIDE);
  for (int bsel = 0; bsel < 2 && ok; bsel++) {
    for (int q = 0; q < 3; q++)
      ok = ok && !dalloc(&c->d_u[bsel][q], slots) && !dalloc(&c->d_v[bsel][q], slots);
    ok = ok && !dalloc(&c->d_sp[bsel], slots) && !dalloc(&c->d_wc[bsel], slots);
    if (c->cfg.track_ids) ok = ok && !dalloc(&c->d_id[bsel], slots);
  }
  ok = ok && !dalloc(&c->d_key, slots) && !dalloc(&c->d_rank, slots) &&
       !dalloc(&c->d_base, nc + 1) && !dalloc(&c->d_cnt, nc) && !dalloc(&c->d_arr, nc) &&
       !dalloc(&c->d_stay, nc) && !dalloc(&c->d_tmp, nc + 1) && !dalloc(&c->d_count, nc + 1) &&
       !dalloc(&c->d_scan_part, (nc + 1) / 1024 + 2) && !dalloc(&c->d_flags, 8);
  ok = ok && cudaMallocHost(&c->h_flags, 8 * sizeof(unsigned long long)) == cudaSuccess;
  ok = ok && !dalloc(&c->d_cellM, (size_t)AMPS_CELLM * nc) && !dalloc(&c->d_cellJ, 24 * nc) &&
       !dalloc(&c->d_energy, 4 + AMPS_GPU_MAX_SPECIES);  // energies, then per-species CFL
  ok = ok && cudaMallocHost(&c->h_energy, 4 * sizeof(double)) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    return false;
  }
  double* zero_v[] = {c->d_En, c->d_Eh, c->d_Bcor_prev, c->d_Bcor_cur};
  for (double* p : zero_v) ok = ok && cudaMemset(p, 0, sizeof(double) * 3 * nv) == cudaSuccess;
  ok = ok && cudaMemset(c->d_Bc, 0, sizeof(double) * 3 * nc) == cudaSuccess;
  if (!c->amr)
    ok = ok && cudaMemset(c->d_J, 0, sizeof(double) * 3 * nc) == cudaSuccess &&
         cudaMemset(c->d_M, 0, sizeof(float) * 243 * nc) == cudaSuccess;
  // cell partials start at zero so an AMR solve before any deposit is defined
  ok = ok && cudaMemset(c->d_cellM, 0, sizeof(float) * AMPS_CELLM * nc) == cudaSuccess &&
       cudaMemset(c->d_cellJ, 0, sizeof(float) * 24 * nc) == cudaSuccess;
  // empty layout: every cell has 8 slack slots
  {
    std::vector<int> base((size_t)nc + 1);
    for (long long i = 0; i <= nc; i++) base[(size_t)i] = (int)(8 * i);
    ok = ok && cudaMemcpy(c->d_base, base.data(), sizeof(int) * (nc + 1), cudaMemcpyHostToDevice) ==
                   cudaSuccess;
  }
  ok = ok && cudaMemset(c->d_cnt, 0, sizeof(int) * nc) == cudaSuccess &&
       cudaMemset(c->d_arr, 0, sizeof(int) * nc) == cudaSuccess &&
       cudaMemset(c->d_stay, 0, sizeof(int) * nc) == cudaSuccess &&
       cudaMemset(c->d_sp[0], 0xFF, (size_t)slots) == cudaSuccess &&
       cudaMemset(c->d_sp[1], 0xFF, (size_t)slots) == cudaSuccess &&
       cudaMemset(c->d_flags, 0, sizeof(unsigned long long) * 8) == cudaSuccess;
  return ok;
}

// slot capacity: particles + 1/4 slack + AMPS_SLACK_MIN slack slots per cell
long long slot_count(long long cap, long long ncell) {
  return cap + cap / 4 + (long long)AMPS_SLACK_MIN * ncell + 1024;
}

template <class T>
bool upload(T** d, const std::vector<T>& h) {
  if (dalloc(d, h.size())) return false;
  return h.empty() ||
         cudaMemcpy(*d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice) == cudaSuccess;
}

// The learned preconditioner's mesh maps (see amps_gpu_ctx::d_pc_in).  The
// interface variant of the output maps hands the corners of every block whose
// region holds a non-free entry to the Jacobi list.
bool upload_pc_maps(amps_gpu_ctx* c, const std::vector<int>& in, const std::vector<int>& out,
                    const std::vector<int>& set, const std::vector<int>& jac, int nsets) {
  c->pc_nsets = nsets;
  c->h_pc_set = set;
  std::vector<int> out1(out), jac1(jac);
  int niface = 0;
  c->h_pc_iface.assign((size_t)c->nb, 0);
  for (int b = 0; b < c->nb; b++) {
    bool iface = false;
    for (int v = 0; v < 1000 && !iface; v++) iface = in[(size_t)b * 1000 + v] < 0;
    if (!iface) continue;
    niface++;
    c->h_pc_iface[(size_t)b] = 1;
    for (int q = 0; q < 512; q++) {
      int& o = out1[(size_t)b * 512 + q];
      if (o >= 0) jac1.push_back(o);
      o = -1;
    }
  }
  c->pc_iface_blocks = niface;
  c->pc_njac_v[0] = (long long)jac.size();
  c->pc_njac_v[1] = (long long)jac1.size();
  const bool ok = upload(&c->d_pc_in, in) && upload(&c->d_pc_out_v[0], out) &&
                  upload(&c->d_pc_jac_v[0], jac) && upload(&c->d_pc_out_v[1], out1) &&
                  upload(&c->d_pc_jac_v[1], jac1) && (nsets == 1 || upload(&c->d_pc_set, set));
  c->d_pc_out = c->d_pc_out_v[0];
  c->d_pc_jac = c->d_pc_jac_v[0];
  c->pc_njac = c->pc_njac_v[0];
  return ok;
}

// Uniform periodic mesh: region corner (i, j, k) in -1..8 of block b is the
// corner of the periodic lattice there; every block writes its 512 corners.
bool build_pc_maps_uniform(amps_gpu_ctx* c) {
  const int nbx = c->cfg.nbx, nby = c->cfg.nby, nbz = c->cfg.nbz;
  const int NX = 8 * nbx, NY = 8 * nby, NZ = 8 * nbz;
  std::vector<int> in((size_t)c->nb * 1000), out((size_t)c->nb * 512), set((size_t)c->nb, 0), jac;
  for (int b = 0; b < c->nb; b++) {
    const int bx = b % nbx, by = (b / nbx) % nby, bz = b / (nbx * nby);
    for (int v = 0; v < 1000; v++) {
      const int I = (8 * bx + v % 10 - 1 + NX) % NX, J = (8 * by + (v / 10) % 10 - 1 + NY) % NY,
                K = (8 * bz + v / 100 - 1 + NZ) % NZ;
      const int ob = (I >> 3) + nbx * ((J >> 3) + nby * (K >> 3));
      in[(size_t)b * 1000 + v] = ob * AMPS_CPB + (I & 7) + 8 * ((J & 7) + 8 * (K & 7));
    }
    for (int q = 0; q < 512; q++) out[(size_t)b * 512 + q] = b * AMPS_CPB + q;
  }
  return upload_pc_maps(c, in, out, set, jac, 1);
}

// AMR mesh: region corner (i, j, k) of block b sits at origin + (i, j, k) *
// scale on the finest lattice (periodic); its entry is the unique corner
// there, -2 - h for a hanging corner h (input interpolated from its parents),
// or -1 where none exists (inside a coarser neighbour's cell).  A free corner
// is written by the block whose cell has it as low corner (the leaf containing
// the corner + (eps, eps, eps)); hanging corners keep z = D v.
bool build_pc_maps_amr(amps_gpu_ctx* c, const amps_amr_mesh* m) {
  const long long nbl = (long long)m->blocks.size(), nv = c->nvc;
  const long long FX = m->nfine[0], FY = m->nfine[1], FZ = m->nfine[2];
  // periodic axes wrap; on open axes positions beyond the faces have no corner
  // (key -1, never stored); corners of open axes run 0..F, hence F + 1 per axis
  const long long SX = FX + 1, SY = FY + 1;
  auto key = [&](long long x, long long y, long long z) -> long long {
    const long long p[3] = {x, y, z}, F[3] = {FX, FY, FZ};
    long long q[3];
    for (int d = 0; d < 3; d++) {
      if (m->open[d]) {
        if (p[d] < 0 || p[d] > F[d]) return -1;
        q[d] = p[d];
      } else {
        q[d] = ((p[d] % F[d]) + F[d]) % F[d];
      }
    }
    return q[0] + SX * (q[1] + SY * q[2]);
  };
  std::unordered_map<long long, int> at;
  at.reserve((size_t)nv * 2);
  for (long long q = 0; q < nv; q++)
    at[key(m->corner_xyz[(size_t)(3 * q)], m->corner_xyz[(size_t)(3 * q + 1)],
           m->corner_xyz[(size_t)(3 * q + 2)])] = (int)q;
  auto hanging = [&](int id) { return m->hang_start[(size_t)id + 1] > m->hang_start[(size_t)id]; };
  std::vector<int> in((size_t)nbl * 1000), out((size_t)nbl * 512), set((size_t)nbl);
  std::vector<char> written((size_t)nv, 0);
  for (long long b = 0; b < nbl; b++) {
    const amps_block_desc& d = m->blocks[(size_t)b];
    const int sc = 1 << (m->lmax - d.level);
    set[(size_t)b] = d.level;
    for (int v = 0; v < 1000; v++) {
      const auto it = at.find(key(d.ix + (long long)(v % 10 - 1) * sc, d.iy + (long long)((v / 10) % 10 - 1) * sc,
                                  d.iz + (long long)(v / 100 - 1) * sc));
      in[(size_t)b * 1000 + v] =
          it == at.end() ? -1 : (hanging(it->second) ? -2 - it->second : it->second);
    }
    for (int q = 0; q < 512; q++) {
      const int id = m->corner_tab[(size_t)b * 729 + (q & 7) + 9 * (((q >> 3) & 7) + 9 * (q >> 6))];
      const bool mine = !hanging(id) && !written[(size_t)id];
      if (mine) written[(size_t)id] = 1;
      out[(size_t)b * 512 + q] = mine ? id : -1;
    }
  }
  std::vector<int> jac;
  for (long long q = 0; q < nv; q++)
    if (!written[(size_t)q]) jac.push_back((int)q);
  return upload_pc_maps(c, in, out, set, jac, m->lmax + 1);
}

}  // namespace

extern "C" {

amps_gpu_status amps_gpu_create(const amps_gpu_config* cfg, amps_gpu_ctx** out) {
  if (!cfg || !out) return AMPS_GPU_INVALID_ARG;
  *out = nullptr;
  if (cfg->nbx <= 0 || cfg->nby <= 0 || cfg->nbz <= 0 || cfg->dx[0] <= 0 || cfg->dx[1] <= 0 ||
      cfg->dx[2] <= 0)
    return AMPS_GPU_INVALID_ARG;
  const long long nbl = (long long)cfg->nbx * cfg->nby * cfg->nbz;
  const long long nc = nbl * 512;
  const long long slots = slot_count(cfg->particle_capacity, nc);
  if (nc > (1LL << 28) || slots > (1LL << 31) - 1) return AMPS_GPU_INVALID_ARG;
  amps_gpu_status cs = check_config(cfg);
  if (cs) return cs;

  amps_gpu_ctx* c = new amps_gpu_ctx();
  c->cfg = *cfg;
  c->nb = (int)nbl;
  c->ncor = nc;
  c->nvc = nc;
  c->cap = cfg->particle_capacity;
  c->slots = slots;
  if (!alloc_context(c)) {
    amps_gpu_destroy(c);
    return AMPS_GPU_CUDA_ERROR;
  }
  // periodic neighbour table
  std::vector<int> nbr((size_t)c->nb * 27);
  for (int b = 0; b < c->nb; b++) {
    const int bx = b % cfg->nbx, by = (b / cfg->nbx) % cfg->nby, bz = b / (cfg->nbx * cfg->nby);
    for (int oz = -1; oz <= 1; oz++)
      for (int oy = -1; oy <= 1; oy++)
        for (int ox = -1; ox <= 1; ox++) {
          const int X = (bx + ox + cfg->nbx) % cfg->nbx, Y = (by + oy + cfg->nby) % cfg->nby,
                    Z = (bz + oz + cfg->nbz) % cfg->nbz;
          nbr[(size_t)b * 27 + nbr_slot(ox, oy, oz)] = X + cfg->nbx * (Y + cfg->nby * Z);
        }
  }
  if (!upload(&c->d_nbr, nbr) || !build_pc_maps_uniform(c)) {
    amps_gpu_destroy(c);
    return AMPS_GPU_CUDA_ERROR;
  }
  *out = c;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_create_amr(const amps_gpu_config* cfg, const amps_amr_mesh* m,
                                    amps_gpu_ctx** out) {
  if (!cfg || !m || !out) return AMPS_GPU_INVALID_ARG;
  *out = nullptr;
  const long long nbl = (long long)m->blocks.size();
  const long long nc = nbl * 512;
  const long long nv = (long long)m->hang_start.size() - 1;
  const long long slots = slot_count(cfg->particle_capacity, nc);
  if (nbl <= 0 || nv <= 0 || nc > (1LL << 28) || slots > (1LL << 31) - 1 ||
      m->corner_tab.size() != (size_t)nbl * 729)
    return AMPS_GPU_INVALID_ARG;
  for (int d = 0; d < 3; d++)
    if (m->nfine[d] <= 0 || m->nfine[d] % 8) return AMPS_GPU_INVALID_ARG;
  amps_gpu_status cs = check_config(cfg);
  if (cs) return cs;

  amps_gpu_ctx* c = new amps_gpu_ctx();
  c->cfg = *cfg;
  // geometry comes from the mesh: level-0 blocks and cell size
  c->cfg.nbx = m->nb0[0];
  c->cfg.nby = m->nb0[1];
  c->cfg.nbz = m->nb0[2];
  for (int d = 0; d < 3; d++) {
    c->cfg.x0[d] = m->x0[d];
    c->cfg.dx[d] = m->dx0;
  }
  c->amr = true;
  c->lmax = m->lmax;
  c->dxf = m->dx0 / (double)(1 << m->lmax);
  c->nb = (int)nbl;
  c->ncor = nc;
  c->nvc = nv;
  c->cap = cfg->particle_capacity;
  c->slots = slots;
  bool ok = alloc_context(c);
  std::vector<int> borg((size_t)nbl * 3), bscale((size_t)nbl);
  std::vector<double> bdx((size_t)nbl);
  std::vector<float> bdtdx((size_t)nbl), binvvol((size_t)nbl);
  // hanging weights split into FP32 pairs for the pair-arithmetic kernels
  std::vector<float> hw_hi(m->hang_weight.size()), hw_lo(m->hang_weight.size());
  for (size_t t = 0; t < hw_hi.size(); t++) {
    hw_hi[t] = (float)m->hang_weight[t];
    hw_lo[t] = (float)(m->hang_weight[t] - (double)hw_hi[t]);
  }
  for (long long b = 0; b < nbl; b++) {
    const amps_block_desc& d = m->blocks[(size_t)b];
    borg[(size_t)(3 * b)] = d.ix;
    borg[(size_t)(3 * b + 1)] = d.iy;
    borg[(size_t)(3 * b + 2)] = d.iz;
    bscale[(size_t)b] = 1 << (m->lmax - d.level);
    bdx[(size_t)b] = m->dx0 / (double)(1 << d.level);
    bdtdx[(size_t)b] = (float)(cfg->dt / bdx[(size_t)b]);
    binvvol[(size_t)b] = (float)(1.0 / (bdx[(size_t)b] * bdx[(size_t)b] * bdx[(size_t)b]));
  }
  ok = ok && upload(&c->d_ctab, m->corner_tab) && upload(&c->d_hs, m->hang_start) &&
       upload(&c->d_hp, m->hang_parent) && upload(&c->d_hw, m->hang_weight) &&
       upload(&c->d_hwh, hw_hi) && upload(&c->d_hwl, hw_lo) &&
       upload(&c->d_fine_map, m->fine_map) && upload(&c->d_borg, borg) &&
       upload(&c->d_bscale, bscale) && upload(&c->d_bdx, bdx) && upload(&c->d_bdtdx, bdtdx) &&
       upload(&c->d_binvvol, binvvol) && build_pc_maps_amr(c, m);
  // identity part of the operator, S = P^T diag(D) P with D(corner) = sum over
  // its cells of V/8: rows of free corners (hanging rows are constraints)
  {
    std::vector<double> D((size_t)nv, 0.0);
    for (long long b = 0; b < nbl; b++) {
      const double v8 = 0.125 * bdx[(size_t)b] * bdx[(size_t)b] * bdx[(size_t)b];
      for (int l = 0; l < 512; l++) {
        const int i = l & 7, j = (l >> 3) & 7, k = l >> 6;
        for (int q = 0; q < 8; q++) {
          const int ci = i + (q & 1), cj = j + ((q >> 1) & 1), ck = k + (q >> 2);
          D[(size_t)m->corner_tab[(size_t)b * 729 + ci + 9 * (cj + 9 * ck)]] += v8;
        }
      }
    }
    std::vector<std::vector<std::pair<int, double>>> rows((size_t)nv);
    auto add = [&](int r, int col, double v) {
      for (auto& e : rows[(size_t)r])
        if (e.first == col) {
          e.second += v;
          return;
        }
      rows[(size_t)r].emplace_back(col, v);
    };
    const auto& hs = m->hang_start;
    for (long long cc = 0; cc < nv; cc++) {
      const int s0 = hs[(size_t)cc], s1 = hs[(size_t)cc + 1];
      if (s0 == s1) {
        add((int)cc, (int)cc, D[(size_t)cc]);
      } else {
        for (int a = s0; a < s1; a++)
          for (int b2 = s0; b2 < s1; b2++)
            add(m->hang_parent[(size_t)a], m->hang_parent[(size_t)b2],
                D[(size_t)cc] * m->hang_weight[(size_t)a] * m->hang_weight[(size_t)b2]);
      }
    }
    std::vector<int> ss((size_t)nv + 1, 0), sc;
    std::vector<double> sv;
    for (long long r = 0; r < nv; r++) {
      ss[(size_t)r] = (int)sc.size();
      if (hs[(size_t)r + 1] > hs[(size_t)r]) continue;  // constraint row
      for (auto& e : rows[(size_t)r]) {
        sc.push_back(e.first);
        sv.push_back(e.second);
      }
    }
    ss[(size_t)nv] = (int)sc.size();
    std::vector<float> svh(sv.size()), svl(sv.size());
    for (size_t q = 0; q < sv.size(); q++) {
      svh[q] = (float)sv[q];
      svl[q] = (float)(sv[q] - (double)svh[q]);
    }
    ok = ok && upload(&c->d_ss, ss) && upload(&c->d_sc, sc) && upload(&c->d_sv, sv) &&
         upload(&c->d_svh, svh) && upload(&c->d_svl, svl);
  }
  if (!ok) {
    cudaGetLastError();
    amps_gpu_destroy(c);
    return AMPS_GPU_CUDA_ERROR;
  }
  // field boundary rows (open axes)
  c->mesh_open = (m->open[0] ? 1 : 0) | (m->open[1] ? 2 : 0) | (m->open[2] ? 4 : 0);
  c->neumann = m->neumann;
  c->open_axes = c->mesh_open;  // particles leave through the open faces
  if (c->mesh_open) {
    std::vector<float> bh(m->bnd_weight.size()), bl(m->bnd_weight.size());
    for (size_t q = 0; q < bh.size(); q++) {
      bh[q] = (float)m->bnd_weight[q];
      bl[q] = (float)(m->bnd_weight[q] - (double)bh[q]);
    }
    ok = upload(&c->d_bflag, m->bnd_flag) && upload(&c->d_bs, m->bnd_start) && upload(&c->d_bc, m->bnd_col) &&
         upload(&c->d_bw, m->bnd_weight) && upload(&c->d_bwh, bh) && upload(&c->d_bwl, bl);
    if (!ok) {
      cudaGetLastError();
      amps_gpu_destroy(c);
      return AMPS_GPU_CUDA_ERROR;
    }
  }
  for (int d = 0; d < 3; d++) c->amrdev.nfine[d] = m->nfine[d];
  c->amrdev.fine_map = c->d_fine_map;
  c->amrdev.borg = c->d_borg;
  c->amrdev.bscale = c->d_bscale;
  c->amrdev.bdtdx = c->d_bdtdx;
  c->amrdev.binvvol = c->d_binvvol;
  *out = c;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_mesh_sizes(const amps_gpu_ctx* c, long long* nblocks, long long* ncells,
                                    long long* ncorners) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  if (nblocks) *nblocks = c->nb;
  if (ncells) *ncells = c->ncor;
  if (ncorners) *ncorners = c->nvc;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_destroy(amps_gpu_ctx* c) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  flush_timers(c);
  staging_free(c);
  precond_free(c->pn);
  c->pn = nullptr;
  species_free(c);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
  for (auto& g : c->solve_graphs) cudaGraphExecDestroy(g.exec);
  c->solve_graphs.clear();
  for (int q = 0; q < 2; q++)
    if (c->arr_ev[q]) cudaEventDestroy(c->arr_ev[q]);
  cudaFree(c->d_dive);
  c->d_dive = nullptr;
  cudaFree(c->d_hstage);
  c->d_hstage = nullptr;
  void* ptrs[] = {c->d_nbr, c->d_En, c->d_Eh, c->d_Bc, c->d_Bc2, c->d_Bcor_prev, c->d_Bcor_cur,
                  c->d_J, c->d_M, c->d_rhs, c->d_x, c->d_V, c->d_w, c->d_dinv, c->d_red, c->d_arn, c->d_xs, c->d_step,
                  c->d_Z, c->d_y32,
                  c->d_stencil_push, c->d_stencil_dep, c->d_stencil_cprev, c->d_stencil_ccur, c->d_key, c->d_rank, c->d_base, c->d_cnt,
                  c->d_arr, c->d_stay, c->d_tmp, c->d_count, c->d_scan_part, c->d_flags,
                  c->d_cellM, c->d_cellJ, c->d_energy, c->d_ctab, c->d_hs, c->d_hp, c->d_hw, c->d_hwh, c->d_hwl,
                  c->d_bflag, c->d_bs, c->d_bc, c->d_bw, c->d_bwh, c->d_bwl,
                  c->d_fine_map, c->d_borg, c->d_bscale, c->d_bdx, c->d_bdtdx, c->d_binvvol,
                  c->d_ss, c->d_sc, c->d_sv, c->d_svh, c->d_svl, c->d_dff, c->d_tmpv, c->d_pc_in, c->d_pc_out_v[0], c->d_pc_out_v[1],
                  c->d_pc_set, c->d_pc_jac_v[0], c->d_pc_jac_v[1]};
  for (void* p : ptrs) cudaFree(p);
  for (int b = 0; b < 2; b++) {
    for (int q = 0; q < 3; q++) {
      cudaFree(c->d_u[b][q]);
      cudaFree(c->d_v[b][q]);
    }
    cudaFree(c->d_sp[b]);
    cudaFree(c->d_wc[b]);
    cudaFree(c->d_id[b]);
  }
  if (c->h_red) cudaFreeHost(c->h_red);
  if (c->h_flags) cudaFreeHost(c->h_flags);
  if (c->h_energy) cudaFreeHost(c->h_energy);
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  for (auto& e : c->copy_ev)
    if (e) cudaEventDestroy(e);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return AMPS_GPU_OK;
}

const char* amps_gpu_last_error(const amps_gpu_ctx* c) { return c ? c->err.c_str() : "null context"; }

amps_gpu_status amps_gpu_get_stream(amps_gpu_ctx* c, void** stream) {
  if (!c || !stream) return AMPS_GPU_INVALID_ARG;
  *stream = (void*)c->stream;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_synchronize(amps_gpu_ctx* c) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  return cuda_check(c, cudaStreamSynchronize(c->stream), "synchronize");
}

amps_gpu_status amps_gpu_import_particles(amps_gpu_ctx* c, long long n, const double* x,
                                          const double* v, const uint8_t* spec,
                                          const double* wcorr) {
  if (!c || n < 0 || (n > 0 && (!x || !v || !spec)))
    return set_err(c, AMPS_GPU_INVALID_ARG, "import_particles: bad arguments");
  if (n > c->cap) return set_err(c, AMPS_GPU_CAPACITY_EXCEEDED, "import_particles: n > capacity");
  cudaSetDevice(c->cfg.device);
  Staging* s = staging(c, std::max(n, 1LL));
  if (!s) return set_err(c, AMPS_GPU_CUDA_ERROR, "import_particles: staging allocation failed");
  c->has_wcorr = wcorr != nullptr;
  amps_gpu_status st = reset_flags(c);
  if (st) return st;
  cudaStream_t q = c->stream;
  if (n > 0) {
    if ((st = cuda_check(c, cudaMemcpyAsync(s->x, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, q), "H2D x")) ||
        (st = cuda_check(c, cudaMemcpyAsync(s->v, v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, q), "H2D v")) ||
        (st = cuda_check(c, cudaMemcpyAsync(s->sp, spec, n, cudaMemcpyHostToDevice, q), "H2D spec")))
      return st;
    if (wcorr && (st = cuda_check(c, cudaMemcpyAsync(s->wc, wcorr, sizeof(double) * n, cudaMemcpyHostToDevice, q), "H2D wcorr")))
      return st;
  }
  st = cuda_check(c, launch_import_fp64(c, s->x, s->v, s->sp, wcorr ? s->wc : nullptr, n), "import");
  if (st) return st;
  c->have_moments = false;
  return check_flags(c, nullptr, nullptr, nullptr);
}

amps_gpu_status amps_gpu_import_particles_local(amps_gpu_ctx* c, long long n, const float* u,
                                                const float* v, const uint8_t* spec,
                                                const int32_t* block) {
  return amps_gpu_import_particles_local_weighted(c, n, u, v, spec, block, nullptr);
}

amps_gpu_status amps_gpu_import_particles_local_weighted(amps_gpu_ctx* c, long long n,
                                                         const float* u, const float* v,
                                                         const uint8_t* spec, const int32_t* block,
                                                         const float* wcorr) {
  if (!c || n < 0 || (n > 0 && (!u || !v || !spec || !block)))
    return set_err(c, AMPS_GPU_INVALID_ARG, "import_particles_local: bad arguments");
  if (n > c->cap) return set_err(c, AMPS_GPU_CAPACITY_EXCEEDED, "import_particles_local: n > capacity");
  cudaSetDevice(c->cfg.device);
  Staging* s = staging(c, std::max(n, 1LL));
  if (!s) return set_err(c, AMPS_GPU_CUDA_ERROR, "staging allocation failed");
  c->has_wcorr = wcorr != nullptr;
  amps_gpu_status st = reset_flags(c);
  if (st) return st;
  cudaStream_t q = c->stream;
  float* du = reinterpret_cast<float*>(s->x);
  float* dv = reinterpret_cast<float*>(s->v);
  float* dw = wcorr ? reinterpret_cast<float*>(s->wc) : nullptr;
  if (n > 0) {
    if ((st = cuda_check(c, cudaMemcpyAsync(du, u, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, q), "H2D u")) ||
        (st = cuda_check(c, cudaMemcpyAsync(dv, v, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, q), "H2D v")) ||
        (st = cuda_check(c, cudaMemcpyAsync(s->sp, spec, n, cudaMemcpyHostToDevice, q), "H2D spec")) ||
        (st = cuda_check(c, cudaMemcpyAsync(s->i0, block, sizeof(int32_t) * n, cudaMemcpyHostToDevice, q), "H2D block")))
      return st;
    if (dw && (st = cuda_check(c, cudaMemcpyAsync(dw, wcorr, sizeof(float) * n, cudaMemcpyHostToDevice, q), "H2D wcorr")))
      return st;
  }
  st = cuda_check(c, launch_import_local(c, du, dv, s->sp, s->i0, dw, n), "import_local");
  if (st) return st;
  c->have_moments = false;
  return check_flags(c, nullptr, nullptr, nullptr);
}

amps_gpu_status amps_gpu_num_particles(amps_gpu_ctx* c, long long* n) {
  if (!c || !n) return AMPS_GPU_INVALID_ARG;
  *n = c->np;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_export_particles(amps_gpu_ctx* c, double* x, double* v, uint8_t* spec,
                                          int32_t* block, int32_t* cell, uint32_t* id,
                                          long long* n) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  if (id && !c->cfg.track_ids) return set_err(c, AMPS_GPU_INVALID_ARG, "export: ids not tracked");
  cudaSetDevice(c->cfg.device);
  const long long np = c->np;
  if (n) *n = np;
  if (np == 0) return AMPS_GPU_OK;
  Staging* s = staging(c, np);
  if (!s) return set_err(c, AMPS_GPU_CUDA_ERROR, "staging allocation failed");
  amps_gpu_status st = cuda_check(
      c, launch_export(c, x ? s->x : nullptr, v ? s->v : nullptr, spec ? s->sp : nullptr,
                       block ? s->i0 : nullptr, cell ? s->i1 : nullptr, id ? s->id : nullptr),
      "export");
  if (st) return st;
  cudaStream_t q = c->stream;
  if (x && (st = cuda_check(c, cudaMemcpyAsync(x, s->x, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, q), "D2H x"))) return st;
  if (v && (st = cuda_check(c, cudaMemcpyAsync(v, s->v, sizeof(double) * 3 * np, cudaMemcpyDeviceToHost, q), "D2H v"))) return st;
  if (block && (st = cuda_check(c, cudaMemcpyAsync(block, s->i0, sizeof(int32_t) * np, cudaMemcpyDeviceToHost, q), "D2H block"))) return st;
  if (cell && (st = cuda_check(c, cudaMemcpyAsync(cell, s->i1, sizeof(int32_t) * np, cudaMemcpyDeviceToHost, q), "D2H cell"))) return st;
  if (spec && (st = cuda_check(c, cudaMemcpyAsync(spec, s->sp, np, cudaMemcpyDeviceToHost, q), "D2H spec"))) return st;
  if (id && (st = cuda_check(c, cudaMemcpyAsync(id, s->id, sizeof(uint32_t) * np, cudaMemcpyDeviceToHost, q), "D2H id"))) return st;
  return cuda_check(c, cudaStreamSynchronize(q), "export sync");
}

amps_gpu_status amps_gpu_import_fields(amps_gpu_ctx* c, const double* E_n, const double* E_half,
                                       const double* B_center, const double* B_corner_prev,
                                       const double* B_corner_cur) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  cudaStreamSynchronize(c->stream);
  amps_gpu_status s;
  const long long nv = c->nvc, nc = c->ncor;
  if ((s = upload_vec3(c, E_n, c->d_En, nv)) || (s = upload_vec3(c, E_half, c->d_Eh, nv)) ||
      (s = upload_vec3(c, B_center, c->d_Bc, nc)) ||
      (s = upload_vec3(c, B_corner_prev, c->d_Bcor_prev, nv)) ||
      (s = upload_vec3(c, B_corner_cur, c->d_Bcor_cur, nv)))
    return s;
  // the centre B^n a centre-B push reads before the first field solve
  return cuda_check(c, cudaMemcpyAsync(c->d_Bc2, c->d_Bc, sizeof(double) * 3 * nc,
                                       cudaMemcpyDeviceToDevice, c->stream), "B centre copy");
}

amps_gpu_status amps_gpu_export_fields(amps_gpu_ctx* c, double* E_n, double* E_half,
                                       double* B_center, double* B_corner_prev,
                                       double* B_corner_cur) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  amps_gpu_status s = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  if (s) return s;
  const long long nv = c->nvc, nc = c->ncor;
  if ((s = download_vec3(c, c->d_En, E_n, nv)) || (s = download_vec3(c, c->d_Eh, E_half, nv)) ||
      (s = download_vec3(c, c->d_Bc, B_center, nc)) ||
      (s = download_vec3(c, c->d_Bcor_prev, B_corner_prev, nv)) ||
      (s = download_vec3(c, c->d_Bcor_cur, B_corner_cur, nv)))
    return s;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_import_moments(amps_gpu_ctx* c, const double* J, const double* M) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  if (c->amr)
    return set_err(c, AMPS_GPU_INVALID_ARG,
                   "import_moments: AMR contexts keep per-cell moments only");
  cudaSetDevice(c->cfg.device);
  cudaStreamSynchronize(c->stream);
  amps_gpu_status s = upload_vec3(c, J, c->d_J, c->ncor);
  if (s) return s;
  if ((s = layout_upload(c, M, c->d_M, c->ncor, 243, true))) return s;
  c->have_moments = true;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_export_moments(amps_gpu_ctx* c, double* J, double* M) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  amps_gpu_status s = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  if (s) return s;
  if (c->amr) return amr_export_corner_moments(c, J, M);
  s = download_vec3(c, c->d_J, J, c->ncor);
  if (s) return s;
  if ((s = layout_download(c, c->d_M, M, c->ncor, 243, true))) return s;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_export_cell_moments(amps_gpu_ctx* c, double* cellJ, double* cellM) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  amps_gpu_status s = cuda_check(c, cudaStreamSynchronize(c->stream), "sync");
  if (s) return s;
  if (!cellJ && !cellM) return AMPS_GPU_OK;
  if ((s = layout_cell_moments(c, cellJ, cellM))) return s;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_move_particles(amps_gpu_ctx* c, long long* out_of_block) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  return particle_step(c, false, out_of_block, nullptr);
}

amps_gpu_status amps_gpu_move_particles_relativistic(amps_gpu_ctx* c, double dt_total,
                                                     double light_speed, long long* substeps) {
  if (!c || !(dt_total >= 0.0) || !(light_speed > 0.0))
    return set_err(c, AMPS_GPU_INVALID_ARG, "move_particles_relativistic: bad arguments");
  cudaSetDevice(c->cfg.device);
  amps_gpu_status s;
  if ((s = reset_flags(c))) return s;
  if ((s = cuda_check(c, launch_relboris(c, c->d_En, c->d_Bcor_cur, dt_total, light_speed, 100000000LL),
                      "relativistic Boris")))
    return s;
  if ((s = cuda_check(c, cudaMemcpyAsync(c->h_flags, c->d_flags, 7 * sizeof(unsigned long long),
                                         cudaMemcpyDeviceToHost, c->stream), "flags")))
    return s;
  if ((s = cuda_check(c, cudaStreamSynchronize(c->stream), "sync"))) return s;
  if (substeps) *substeps = (long long)c->h_flags[5];
  // particles that left through an open face were not placed
  c->np -= (long long)c->h_flags[6];
  c->deleted_total += (long long)c->h_flags[6];
  if (c->h_flags[2])
    return set_err(c, AMPS_GPU_DEVICE_TIMEOUT, "relativistic Boris: sub-step cap reached");
  c->have_moments = false;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_move_particles_boris(amps_gpu_ctx* c, double dt_total) {
  if (!c || !(dt_total >= 0.0))
    return set_err(c, AMPS_GPU_INVALID_ARG, "move_particles_boris: bad arguments");
  cudaSetDevice(c->cfg.device);
  amps_gpu_status s;
  if ((s = reset_flags(c))) return s;
  if ((s = cuda_check(c, launch_relboris(c, c->d_En, c->d_Bcor_cur, dt_total, 1.0, 1, false),
                      "Boris")))
    return s;
  if ((s = cuda_check(c, cudaMemcpyAsync(c->h_flags, c->d_flags, 7 * sizeof(unsigned long long),
                                         cudaMemcpyDeviceToHost, c->stream), "flags")))
    return s;
  if ((s = cuda_check(c, cudaStreamSynchronize(c->stream), "sync"))) return s;
  // particles that left through an open face were not placed
  c->np -= (long long)c->h_flags[6];
  c->deleted_total += (long long)c->h_flags[6];
  c->have_moments = false;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_update_j_mass_matrix(amps_gpu_ctx* c, double* particle_energy) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  amps_gpu_status s;
  if ((s = reset_flags(c))) return s;
  if ((s = cuda_check(c, launch_pack_stencils(c, c->d_Eh, c->d_Bcor_prev, c->d_Bcor_cur), "pack")))
    return s;
  if ((s = cuda_check(c, launch_deposit(c), "deposit"))) return s;
  if ((s = cuda_check(c, launch_species_moments(c), "species moments"))) return s;
  if ((s = cuda_check(c, cudaMemcpyAsync(c->h_energy, c->d_energy, sizeof(double),
                                         cudaMemcpyDeviceToHost, c->stream), "energy")))
    return s;
  if ((s = check_flags(c, nullptr, nullptr, nullptr))) return s;
  if (particle_energy) *particle_energy = c->h_energy[0];
  c->have_moments = true;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_push_deposit(amps_gpu_ctx* c, double* particle_energy) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  amps_gpu_status s = particle_step(c, true, nullptr, nullptr);
  if (s) return s;
  if (particle_energy) {
    if ((s = cuda_check(c, cudaMemcpy(c->h_energy, c->d_energy, sizeof(double),
                                      cudaMemcpyDeviceToHost), "energy")))
      return s;
    *particle_energy = c->h_energy[0];
  }
  c->have_moments = true;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_field_solve(amps_gpu_ctx* c, double tol, int maxit, int precond,
                                     amps_gpu_solve_stats* stats) {
  if (!c || tol <= 0.0 || maxit <= 0 || precond < 0 || precond > 2)
    return set_err(c, AMPS_GPU_INVALID_ARG, "field_solve: bad arguments");
  cudaSetDevice(c->cfg.device);
  amps_gpu_status s;
  amps_gpu_solve_stats st{};
  // the tensor-core preconditioner and the AMR operator's staged copies
  // report bounded-wait timeouts in the flags
  const bool watch = precond == 2 || c->amr;
  if (watch && (s = reset_flags(c))) return s;
  if ((s = cuda_check(c, launch_rhs(c), "rhs"))) return s;
  amps_gpu_status gs = gmres_solve(c, tol, maxit, precond, &st);
  if (gs != AMPS_GPU_OK && gs != AMPS_GPU_GMRES_NOT_CONVERGED) return gs;
  if (watch && (s = check_flags(c, nullptr, nullptr, nullptr))) return s;
  // ProcessFinalSolution: E^{n+theta} = E^n + dE
  if ((s = cuda_check(c, launch_add(c, c->d_En, c->d_x, c->d_Eh, 3 * c->nvc), "E_half"))) return s;
  if ((s = cuda_check(c, launch_update_b(c), "update_b"))) return s;
  std::swap(c->d_Bc, c->d_Bc2);
  std::swap(c->d_Bcor_prev, c->d_Bcor_cur);
  if ((s = cuda_check(c, launch_c2n(c, c->d_Bc, c->d_Bcor_cur), "c2n"))) return s;
  if ((s = cuda_check(c, launch_update_e(c), "update_e"))) return s;
  if ((s = cuda_check(c, cudaMemcpyAsync(c->h_energy + 1, c->d_energy + 1, sizeof(double),
                                         cudaMemcpyDeviceToHost, c->stream), "wave energy")))
    return s;
  if ((s = cuda_check(c, cudaStreamSynchronize(c->stream), "sync"))) return s;
  st.wave_energy = c->h_energy[1];
  if (stats) *stats = st;
  if (gs == AMPS_GPU_GMRES_NOT_CONVERGED)
    return set_err(c, gs, "GMRES did not converge: iterations " + std::to_string(st.iterations) +
                              ", relative residual " + std::to_string(st.rel_residual));
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_step(amps_gpu_ctx* c, double tol, int maxit, int precond,
                              amps_gpu_step_stats* stats) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  amps_gpu_status s;
  amps_gpu_step_stats st{};
  if (!c->have_moments) {
    if ((s = amps_gpu_update_j_mass_matrix(c, nullptr))) return s;
  }
  amps_gpu_status fs = amps_gpu_field_solve(c, tol, maxit, precond, &st.solve);
  if (fs != AMPS_GPU_OK && fs != AMPS_GPU_GMRES_NOT_CONVERGED) return fs;
  if ((s = particle_step(c, true, &st.out_of_block, &st.ulp_face))) return s;
  if ((s = cuda_check(c, cudaMemcpy(c->h_energy, c->d_energy, sizeof(double),
                                    cudaMemcpyDeviceToHost), "energy")))
    return s;
  st.particle_energy = c->h_energy[0];
  c->have_moments = true;
  if (stats) *stats = st;
  return fs;
}

amps_gpu_status amps_gpu_set_open_axes(amps_gpu_ctx* c, int open_x, int open_y, int open_z) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  cudaStreamSynchronize(c->stream);
  const int want = (open_x ? 1 : 0) | (open_y ? 2 : 0) | (open_z ? 4 : 0);
  // an AMR mesh without periodic wrap on an axis has no particle wrap there either
  if (c->amr && c->mesh_open && want != c->mesh_open)
    return set_err(c, AMPS_GPU_INVALID_ARG, "set_open_axes: the mesh fixes the open axes");
  c->open_axes = want;
  // captured particle steps carry the old setting in their kernel arguments
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_add_injection(amps_gpu_ctx* c, int face, int spec, double density,
                                       const double* drift, double vth) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  if (face < 0 || face > 5 || !((c->open_axes >> (face >> 1)) & 1))
    return set_err(c, AMPS_GPU_INVALID_ARG, "add_injection: the face must belong to an open axis");
  if (spec < 0 || spec >= c->cfg.nspec || !(vth > 0.0) || !(density >= 0.0) || c->inj.size() >= 8)
    return set_err(c, AMPS_GPU_INVALID_ARG, "add_injection: bad species, density, vth or too many sources");
  cudaSetDevice(c->cfg.device);
  cudaStreamSynchronize(c->stream);
  if (!c->d_step) {
    unsigned long long init[2] = {0ull, (unsigned long long)c->next_id};
    if (cudaMalloc(reinterpret_cast<void**>(&c->d_step), sizeof(init)) != cudaSuccess ||
        cudaMemcpy(c->d_step, init, sizeof(init), cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      return set_err(c, AMPS_GPU_CUDA_ERROR, "add_injection: allocation failed");
    }
  }
  amps_gpu_ctx::InjSource s;
  s.face = face;
  s.spec = spec;
  s.density = density;
  for (int d = 0; d < 3; d++) s.drift[d] = drift ? drift[d] : 0.0;
  s.vth = vth;
  c->inj.push_back(s);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_clear_injection(amps_gpu_ctx* c) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  cudaStreamSynchronize(c->stream);
  c->inj.clear();
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_set_injection_seed(amps_gpu_ctx* c, unsigned long long seed) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  c->inj_seed = seed;
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
  c->graphs.clear();
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_injected_particles(amps_gpu_ctx* c, long long* total) {
  if (!c || !total) return AMPS_GPU_INVALID_ARG;
  *total = c->injected_total;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_deleted_particles(amps_gpu_ctx* c, long long* total) {
  if (!c || !total) return AMPS_GPU_INVALID_ARG;
  *total = c->deleted_total;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_set_graphs(amps_gpu_ctx* c, int on) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  c->use_graphs = on != 0;
  return AMPS_GPU_OK;
}

// the field kernels' launch shapes now, on scratch vectors; the arrivals chunk
// over the next particle steps (3 with each variant), which do their work as
// usual
amps_gpu_status amps_gpu_autotune(amps_gpu_ctx* c, double* ms) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  cudaSetDevice(c->cfg.device);
  for (int q = 0; q < 2; q++)
    if (!c->arr_ev[q] && cudaEventCreate(&c->arr_ev[q]) != cudaSuccess)
      return set_err(c, AMPS_GPU_CUDA_ERROR, "autotune: event creation failed");
  c->arr_tune_left = 6;
  c->arr_tune_ms[0] = c->arr_tune_ms[1] = 0.0;
  c->arr_tune_n[0] = c->arr_tune_n[1] = 0;
  return field_autotune(c, ms);
}

amps_gpu_status amps_gpu_set_b_center(amps_gpu_ctx* c, int on) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  if (on && c->amr)
    return set_err(c, AMPS_GPU_INVALID_ARG, "set_b_center: centre B is built for uniform meshes");
  cudaSetDevice(c->cfg.device);
  if (on && !c->d_stencil_cprev) {
    const size_t n = (size_t)c->nb * AMPS_CSC * 4;
    if (dalloc(&c->d_stencil_cprev, n) || dalloc(&c->d_stencil_ccur, n))
      return set_err(c, AMPS_GPU_CUDA_ERROR, "set_b_center: centre stencils");
  }
  c->b_center = on != 0;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_set_arrivals_chunk(amps_gpu_ctx* c, int chunk) {
  if (!c || (chunk != 16 && chunk != 32)) return set_err(c, AMPS_GPU_INVALID_ARG, "arrivals chunk: 16 or 32");
  c->arr_chunk = chunk;
  c->arr_tune_left = 0;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_get_particle_tuning(amps_gpu_ctx* c, int* arrivals_chunk, int* pending,
                                             double* ms) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  if (arrivals_chunk) *arrivals_chunk = c->arr_chunk;
  if (pending) *pending = c->arr_tune_left;
  for (int q = 0; ms && q < 2; q++) ms[q] = c->arr_tune_n[q] ? c->arr_tune_ms[q] / c->arr_tune_n[q] : 0.0;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_get_tuning(amps_gpu_ctx* c, int* threads_per_cta, int* reduction_ctas) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  if (threads_per_cta) *threads_per_cta = c->tune_tb;
  if (reduction_ctas) *reduction_ctas = c->tune_red;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_set_kernel_timing(amps_gpu_ctx* c, int enable) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  flush_timers(c);
  c->timing = enable != 0;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_get_kernel_times(amps_gpu_ctx* c, const char** names, double* total_ms,
                                          long long* launches, int cap, int* n) {
  if (!c || !n) return AMPS_GPU_INVALID_ARG;
  flush_timers(c);
  int k = 0;
  for (auto& t : c->timers) {
    if (k >= cap) break;
    if (names) names[k] = t.name;
    if (total_ms) total_ms[k] = t.ms;
    if (launches) launches[k] = t.launches;
    k++;
  }
  *n = k;
  return AMPS_GPU_OK;
}

amps_gpu_status amps_gpu_reset_kernel_times(amps_gpu_ctx* c) {
  if (!c) return AMPS_GPU_INVALID_ARG;
  flush_timers(c);
  for (auto& t : c->timers) {
    t.ms = 0.0;
    t.launches = 0;
  }
  return AMPS_GPU_OK;
}

}  // extern "C"
