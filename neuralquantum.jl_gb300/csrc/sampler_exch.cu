// FP32 exchange-rule instantiations of the Metropolis sampler (see sampler_impl.cuh).
#include "sampler_impl.cuh"

cudaError_t launch_rbm_sampler_exchange(const RbmDev<float>& net, const SamplerRun& run, int G, cudaStream_t st) {
  if (net.n_rows < 1 || net.n_half != 0) return cudaErrorInvalidValue;
  if (net.act == ACT_LOGCOSH) return sampler_g<float, ACT_LOGCOSH, true>(net, run, G, st);
  return sampler_g<float, ACT_SOFTPLUS, true>(net, run, G, st);
}
