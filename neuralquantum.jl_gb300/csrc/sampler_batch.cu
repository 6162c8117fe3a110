// FP32 instantiation of the many-problem sampler launch.
#include "sampler_impl.cuh"

template cudaError_t launch_rbm_sampler_batch<float>(const SamplerJob<float>*, const int*, int, int, int, int, int,
                                                     int, cudaStream_t);
