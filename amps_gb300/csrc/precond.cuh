// State of the learned preconditioner (precond.cu, precond_tc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

struct amps_gpu_ctx;

extern const int kWSize[3];  // weights per layer: 27*3*32, 27*32*32, 27*32*3

// Weight sets: one network per refinement level of the mesh (one set on a
// uniform mesh).  w/g/m/v point at the active set inside the per-layer
// storage wb/gb/mb/vb ([nsets][kWSize[l]]); load, get, train, loss_grad and
// the sample-mode forward act on the active set, mesh inference uses every
// block's own set.
struct PrecondState {
  float* w[3] = {nullptr, nullptr, nullptr};  // FP32 masters [27][cin][cout]
  float* g[3] = {nullptr, nullptr, nullptr};  // gradients
  float* m[3] = {nullptr, nullptr, nullptr};  // Adam moments
  float* v[3] = {nullptr, nullptr, nullptr};
  float* wb[3] = {nullptr, nullptr, nullptr};
  float* gb[3] = {nullptr, nullptr, nullptr};
  float* mb[3] = {nullptr, nullptr, nullptr};
  float* vb[3] = {nullptr, nullptr, nullptr};
  int nsets = 1, active = 0;
  long long adam_t = 0;
  std::vector<long long> adam_saved;
  // BF16 operand images of the weights for the tensor-core kernel, one per
  // set (each bulk-copied into shared memory by the CTAs of its blocks)
  uint16_t* wtc = nullptr;
  bool tc_ready = false;
  bool use_tc = false;
  // harvested samples: sx[cap][1000][3], se[cap][512][3], and each sample's
  // weight set (the level of the block it came from)
  float* sx = nullptr;
  float* se = nullptr;
  long long cap = 0, n = 0;
  std::vector<int> sample_set;
  std::vector<char> sample_iface;  // sample's block reaches a refinement interface
  // work buffers for S samples
  int work_S = 0;
  float *wx = nullptr, *we = nullptr, *h1 = nullptr, *h2 = nullptr, *y = nullptr;
  float *dy = nullptr, *dh1 = nullptr, *dh2 = nullptr, *wt = nullptr;
  int* perm = nullptr;
  long long perm_n = 0;
  double* dloss = nullptr;  // device loss accumulator
  unsigned long long* flags = nullptr;  // the context's device flags ([2]: timeouts)
};

void precond_select(PrecondState* P, int set);
cudaError_t precond_work(PrecondState* P, int S);
void precond_free(PrecondState* P);
cudaError_t precond_forward32(PrecondState* P, cudaStream_t st, int S);
cudaError_t precond_backward32(PrecondState* P, cudaStream_t st, int S, double* d_loss);
cudaError_t precond_zero_grads(PrecondState* P, cudaStream_t st);
cudaError_t precond_adam(PrecondState* P, cudaStream_t st, float lr);
cudaError_t precond_gather_batch(PrecondState* P, cudaStream_t st, int S, long long first);
cudaError_t precond_owned_out(PrecondState* P, cudaStream_t st, int S, float* out);
// BF16 tcgen05 inference: x[S][1000][3] -> y[S][1000][3] (owned voxels), active set
cudaError_t precond_prepare_tc(PrecondState* P, cudaStream_t st);
cudaError_t precond_forward_tc(PrecondState* P, cudaStream_t st, int S, const float* x, float* y);
// z = D v + N(D v) on the corners the blocks write, in one launch (gather
// through in_map, network with the block's weight set, scatter through out_map)
cudaError_t precond_apply_tc_mesh(PrecondState* P, cudaStream_t st, int nb, const int* in_map,
                                  const int* hs, const int* hp, const double* hw,
                                  const int* out_map, const int* set, long long nvc,
                                  const double* v, const double* dinv, double* z);
// GMRES hooks (field.cu)
cudaError_t launch_precond_net(amps_gpu_ctx* c, const double* v, double* z);
cudaError_t precond_harvest_pairs(amps_gpu_ctx* c, const double* r, const double* e, int e_scaled);
