// FP64 instantiations of the Metropolis sampler with units at weight 1/2
// (the λ units of a density matrix; see sampler_impl.cuh).
#include "sampler_impl.cuh"

template <typename R>
cudaError_t launch_rbm_sampler_half(const RbmDev<R>& net, const SamplerRun& run, int G, cudaStream_t st) {
  if (net.N > 64 || net.M > 320 || !hpl_ok((net.M + G - 1) / G)) return cudaErrorInvalidValue;
  if (net.act == ACT_LOGCOSH) return sampler_g<R, ACT_LOGCOSH, false, true>(net, run, G, st);
  return sampler_g<R, ACT_SOFTPLUS, false, true>(net, run, G, st);
}

template cudaError_t launch_rbm_sampler_half<double>(const RbmDev<double>&, const SamplerRun&, int, cudaStream_t);
