// FP32 instantiations of the Metropolis sampler (see sampler_impl.cuh).
#include "sampler_impl.cuh"

int rbm_sampler_valid_lanes(int N, int M, int csize, int* out, int max_out) {
  const int cand[4] = {4, 8, 16, 32};
  int n = 0;
  for (int c : cand) {
    const int hpl = (M + c - 1) / c;
    // tables of the padded units must fit the 227 KiB of opt-in shared memory
    const size_t smem = (size_t)4 * N * (c * hpl) * csize + (size_t)N * csize / 2;
    if (hpl_ok(hpl) && smem <= 232448 && n < max_out) out[n++] = c;
  }
  return n;
}

template cudaError_t launch_rbm_sampler<float>(const RbmDev<float>&, const SamplerRun&, int, cudaStream_t);
