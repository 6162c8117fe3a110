// tcgen05 (5th-generation tensor core) kernels for sm_103a.
#include "nq_kernels.cuh"

int gram_tc_supported() { return 0; }

cudaError_t launch_gram_tc(const float* X, int rows, int Ns_pad, int split3, float* G,
                           float* partial, int ksplit, cudaStream_t st) {
  (void)X; (void)rows; (void)Ns_pad; (void)split3; (void)G; (void)partial; (void)ksplit; (void)st;
  return cudaErrorNotSupported;
}
