// FP64 instantiations of the Metropolis sampler (see sampler_impl.cuh).
#include "sampler_impl.cuh"

template cudaError_t launch_rbm_sampler<double>(const RbmDev<double>&, const SamplerRun&, int, cudaStream_t);
