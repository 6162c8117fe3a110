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

// Scratch of the statistics kernels: the per-block summaries of launch_stats
// (5 doubles per block of 64 chains), 40 KiB per device at the maximum chain
// count.  Every word a call reads is written earlier in the same call, so
// nothing has to start at zero.
constexpr size_t kScratchDoubles = stats_scratch_doubles(kMaxChains);
static_assert(kScratchDoubles == 5 * ((kMaxChains + 63) / 64), "scratch follows launch_stats' block layout");
static __device__ __align__(256) double g_chain_scratch[kScratchDoubles];

// Device address of g_chain_scratch, looked up once per device and context.
// The address belongs to the module loaded in the device's current context:
// after cudaDeviceReset (or any teardown of the primary context) the module is
// loaded again and the symbol may move, so the cache is keyed by the context's
// unique id (cuCtxGetId, reached through the runtime's driver entry points);
// without that entry point the address is looked up on every call.
struct ScratchSlot {
  unsigned long long ctx_id = 0;
  double* ptr = nullptr;
};
std::mutex g_mu;
ScratchSlot g_slot[kMaxDevices];

typedef int (*PFN_ctx_get_current)(void** ctx);
typedef int (*PFN_ctx_get_id)(void* ctx, unsigned long long* id);

bool current_context_id(unsigned long long* id) {
  static PFN_ctx_get_current get_current = nullptr;
  static PFN_ctx_get_id get_id = nullptr;
  static bool looked = false;
  if (!looked) {
    looked = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<PFN_ctx_get_current>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<PFN_ctx_get_id>(p);
    cudaGetLastError();
  }
  if (!get_current || !get_id) return false;
  void* ctx = nullptr;
  if (get_current(&ctx) != 0 || !ctx) return false;
  return get_id(ctx, id) == 0;
}

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
    unsigned long long ctx_id = 0;
    const bool have_id = current_context_id(&ctx_id);
    ScratchSlot& slot = g_slot[dev];
    if (!have_id || !slot.ptr || slot.ctx_id != ctx_id) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_chain_scratch);
      if (e != cudaSuccess) {
        snprintf(msg, sizeof(msg), "nq_measurement_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
        set_err(err, err_len, msg);
        return NQ_ERR_CUDA;
      }
      slot.ptr = static_cast<double*>(p);
      slot.ctx_id = have_id ? ctx_id : 0;
    }
    scratch = slot.ptr;
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
