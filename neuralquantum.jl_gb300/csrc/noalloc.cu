// nq_measurement_noalloc: the chain statistics of nq_estimate (per-chain
// mean/variance pass, then the Measurement pass) on caller-owned device
// values, with the per-chain scratch taken from a fixed file-scope device
// array instead of a handle's allocation.  Nothing here calls cudaMalloc,
// cudaFree or any allocating library routine.
#include <cstdio>
#include <mutex>

#include "../../include/nqcuda.h"
#include "nq_kernels.cuh"

namespace {

constexpr int kMaxChains = NQ_NOALLOC_MAX_CHAINS;
constexpr int kMaxDevices = 64;

// Scratch of the statistics kernels (4 doubles per 64 chains; sized by the
// 3B + 4 bound that launch_stats documents, 1.5 MiB per device).  Every word
// a call reads is written earlier in the same call, so nothing has to start
// at zero.
static __device__ __align__(256) double g_chain_scratch[3 * kMaxChains];

std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {};

void set_err(char* err, size_t len, const char* msg) {
  if (err && len > 0) snprintf(err, len, "%s", msg);
}

bool device_accessible(const void* p, int dev) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type == cudaMemoryTypeManaged) return true;
  return a.type == cudaMemoryTypeDevice && a.device == dev;
}

}  // namespace

extern "C" nq_status nq_measurement_noalloc(const void* d_values, int32_t dtype, int32_t n_chains,
                                            int32_t chain_length, int32_t kind, double* d_out6, void* stream,
                                            char* err, size_t err_len) {
  char msg[256];
  if (!d_values || !d_out6) {
    set_err(err, err_len, "nq_measurement_noalloc: d_values and d_out6 must be device pointers");
    return NQ_ERR_ARG;
  }
  if (dtype != NQ_DTYPE_C64 && dtype != NQ_DTYPE_C128) {
    set_err(err, err_len, "nq_measurement_noalloc: dtype must be NQ_DTYPE_C64 or NQ_DTYPE_C128");
    return NQ_ERR_ARG;
  }
  if (kind != 0 && kind != 1) {
    set_err(err, err_len, "nq_measurement_noalloc: kind must be 0 (values) or 1 (squared modulus)");
    return NQ_ERR_ARG;
  }
  if (n_chains < 1 || chain_length < 1) {
    set_err(err, err_len, "nq_measurement_noalloc: n_chains and chain_length must be >= 1");
    return NQ_ERR_ARG;
  }
  if (n_chains > kMaxChains) {
    snprintf(msg, sizeof(msg),
             "nq_measurement_noalloc: n_chains = %d exceeds the fixed scratch of %d chains; "
             "use nq_estimate on a handle instead",
             n_chains, kMaxChains);
    set_err(err, err_len, msg);
    return NQ_ERR_ARG;
  }
  const size_t esz = dtype == NQ_DTYPE_C64 ? 8 : 16;
  if ((reinterpret_cast<uintptr_t>(d_values) % (esz / 2)) != 0 || (reinterpret_cast<uintptr_t>(d_out6) % 8) != 0) {
    set_err(err, err_len, "nq_measurement_noalloc: misaligned d_values or d_out6");
    return NQ_ERR_ARG;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    set_err(err, err_len, "nq_measurement_noalloc: no usable current CUDA device");
    return NQ_ERR_CUDA;
  }
  if (!device_accessible(d_values, dev) || !device_accessible(d_out6, dev)) {
    set_err(err, err_len, "nq_measurement_noalloc: d_values and d_out6 must be memory of the current device");
    return NQ_ERR_ARG;
  }
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_chain_scratch);
      if (e != cudaSuccess) {
        snprintf(msg, sizeof(msg), "nq_measurement_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        set_err(err, err_len, msg);
        return NQ_ERR_CUDA;
      }
      g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    scratch = g_scratch_ptr[dev];
  }
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == NQ_DTYPE_C64)
    e = launch_stats<float>(static_cast<const cpx<float>*>(d_values), n_chains, chain_length, kind, scratch,
                            d_out6, st);
  else
    e = launch_stats<double>(static_cast<const cpx<double>*>(d_values), n_chains, chain_length, kind, scratch,
                             d_out6, st);
  if (e != cudaSuccess) {
    snprintf(msg, sizeof(msg), "nq_measurement_noalloc: launch failed: %s", cudaGetErrorString(e));
    set_err(err, err_len, msg);
    return NQ_ERR_CUDA;
  }
  set_err(err, err_len, "");
  return NQ_OK;
}
