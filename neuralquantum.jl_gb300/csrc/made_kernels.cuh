// Launch interfaces of the learned autoregressive proposal (MADE).
#pragma once
#include <cuda_bf16.h>

#include "nq_kernels.cuh"

// Inference view: BF16 weights laid out for warp access, FP32 biases.
struct MadeDev {
  int N = 0, H = 128;
  const __nv_bfloat16* W1T = nullptr;   // [N][H]
  const __nv_bfloat16* W2T = nullptr;   // [H][H], W2T[k'][k] = W2[k][k']
  const __nv_bfloat16* W3 = nullptr;    // [N][H]
  const float* b1 = nullptr;            // [H]
  const float* b2 = nullptr;            // [H]
  const float* b3 = nullptr;            // [N]
};
// writable alias used by the pack kernel
struct MadeDevW {
  __nv_bfloat16 *W1T, *W2T, *W3;
  float *b1, *b2, *b3;
};

// Training view: FP32 master (flat W1 [H][N], b1, W2 [H][H], b2, W3 [N][H], b3),
// Adam moments and the autoregressive mask.
struct MadeTrain {
  int N = 0, H = 128, n_params = 0;
  float* master = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  const float* mask = nullptr;
};

int made_n_params(int N, int H);
cudaError_t launch_made_mask(int N, int H, float* mask, cudaStream_t st);
cudaError_t launch_made_apply_mask(int n_params, const float* mask, float* master, cudaStream_t st);
cudaError_t launch_made_pack(const MadeDev& m, const float* master, cudaStream_t st);
cudaError_t launch_made_logq(const MadeDev& m, const uint64_t* x, int n, float* out, cudaStream_t st);
// proposals for `slots` AR steps of every chain, Philox stream TAG_AR; the
// call index is read from call_ptr when it is given (graph replays)
cudaError_t launch_made_sample(const MadeDev& m, int n_chains, int slots, uint32_t call, uint32_t k0, uint32_t k1,
                               uint64_t* xout, float* lqout, cudaStream_t st, const uint32_t* call_ptr = nullptr);
// samples per block of the gradient kernel; partial needs ceil(n/chunk)*n_params floats
int made_grad_chunk();
// masked gradient of the mean NLL of x[0..n) into grad (n_params floats)
cudaError_t launch_made_grad(const MadeTrain& t, const uint64_t* x, int n, float* partial, float* grad,
                             cudaStream_t st);
// one Adam step (step >= 1) of the master on grad
cudaError_t launch_made_adam(const MadeTrain& t, const float* grad, float lr, int step, cudaStream_t st);

// Mixture sampler (local flips + learned independent proposals), FP32 RBM.
struct MixParams {
  MadeDev made;
  unsigned long long thr = 0;              // AR move iff TAG_MIX word < thr (= ceil(p_ar 2^32))
  unsigned long long* ar_stats = nullptr;  // [2]: AR proposals, accepted AR proposals (added to)
  // proposals drawn ahead of the chain kernel (launch_made_sample with the same
  // call and key): slot k of chain c at c * pre_slots + k; slots past
  // pre_slots are drawn inside the chain kernel
  const uint64_t* pre_x = nullptr;
  const float* pre_lq = nullptr;
  int pre_slots = 0;
};
bool mix_sampler_supported(int N, int M, int n_half, int H);
cudaError_t launch_rbm_mix_sampler(const RbmDev<float>& net, const SamplerRun& run, const MixParams& mix,
                                   cudaStream_t st);
