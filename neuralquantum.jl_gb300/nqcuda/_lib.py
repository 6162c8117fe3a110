"""ctypes binding of libnqcuda (include/nqcuda.h) and its in-tree build.

The shared library is built in-tree into ``nqcuda/_build/libnqcuda.so`` by
:func:`build` (nvcc for sm_103a).  :func:`lib` loads it and raises if it is
missing: there is no CPU fallback for the engine.
"""
import ctypes
import os
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

_PKG = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_PKG)                       # neuralquantum.jl_gb300/
_REPO = os.path.dirname(_ROOT)
CSRC = os.path.join(_ROOT, "csrc")
INCLUDE = os.path.join(_REPO, "include")
BUILD_DIR = os.path.join(_PKG, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libnqcuda.so")
SOURCES = ["api.cu", "rbm.cu", "sampler_f32.cu", "sampler_f64.cu", "sr.cu", "tc.cu", "spdinv.cu", "ndm.cu",
           "made.cu", "mix_sampler.cu", "proposal.cu", "noalloc.cu", "sampler_batch.cu", "theta_tc.cu",
           "srcg.cu", "exact.cu", "sampler_exch.cu", "sampler_oprule.cu", "chain.cu",
           "sampler_half32.cu", "sampler_half64.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"]

NQ_OK, NQ_ERR_ARG, NQ_ERR_CUDA, NQ_ERR_NOT_PD, NQ_ERR_TIMEOUT, NQ_ERR_NAN, NQ_ERR_STATE, \
    NQ_ERR_UNSUPPORTED = range(8)
STATUS_NAMES = ["NQ_OK", "NQ_ERR_ARG", "NQ_ERR_CUDA", "NQ_ERR_NOT_PD", "NQ_ERR_TIMEOUT",
                "NQ_ERR_NAN", "NQ_ERR_STATE", "NQ_ERR_UNSUPPORTED"]
NQ_NET_RBM, NQ_NET_NDM, NQ_NET_RBM_SPLIT, NQ_NET_NDM_SYMM, NQ_NET_CHAIN, NQ_NET_MIXED_CHAIN = 0, 1, 2, 3, 4, 5
NQ_LAYER_DENSE, NQ_LAYER_WSUM, NQ_LAYER_SUM, NQ_LAYER_DENSE_SPLIT, NQ_LAYER_POSITIVE_DEF_R = 0, 1, 2, 3, 4
NQ_ACT_LOGCOSH, NQ_ACT_SOFTPLUS, NQ_ACT_IDENTITY = 0, 1, 2
NQ_HILB_SPIN, NQ_HILB_FOCK = 0, 1
NQ_DTYPE_C64, NQ_DTYPE_C128, NQ_DTYPE_F32, NQ_DTYPE_F64 = 0, 1, 2, 3
NQ_EVAL_F32, NQ_EVAL_TC_BF16X2, NQ_EVAL_F64, NQ_EVAL_TC_BF16X3 = 0, 1, 2, 3
NQ_S_F32, NQ_S_TF32, NQ_S_TF32X3, NQ_S_F64, NQ_S_BF16 = 0, 1, 2, 3, 4
NQ_SR_DIRECT, NQ_SR_CG = 0, 1
NQ_SAMPLER_METROPOLIS, NQ_SAMPLER_EXACT = 0, 1
NQ_RULE_LOCAL, NQ_RULE_EXCHANGE, NQ_RULE_OPERATOR = 0, 1, 2
NQ_SPACE_NETWORK, NQ_SPACE_DIAGONAL = 0, 1
NQ_QUIRK_STALE_LAST_SLOT = 0x1


class NqConfig(ctypes.Structure):
    _fields_ = [("network", ctypes.c_int32), ("activation", ctypes.c_int32),
                ("hilbert", ctypes.c_int32), ("n_sites", ctypes.c_int32),
                ("n_hidden", ctypes.c_int32), ("n_ancilla", ctypes.c_int32),
                ("n_chains", ctypes.c_int32), ("chain_length", ctypes.c_int32),
                ("burn", ctypes.c_int32), ("passes", ctypes.c_int32),
                ("seed", ctypes.c_uint64), ("eval_precision", ctypes.c_int32),
                ("s_precision", ctypes.c_int32), ("quirks", ctypes.c_uint32),
                ("sampler_lanes", ctypes.c_int32), ("sr_algorithm", ctypes.c_int32),
                ("sampler_kind", ctypes.c_int32), ("rule", ctypes.c_int32), ("sampler_space", ctypes.c_int32),
                ("n_symm", ctypes.c_int32), ("reserved", ctypes.c_int32 * 1)]


class NqLayer(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("n_in", ctypes.c_int32), ("n_out", ctypes.c_int32),
                ("activation", ctypes.c_int32)]


class NqMeasurement(ctypes.Structure):
    _fields_ = [("mean_re", ctypes.c_double), ("mean_im", ctypes.c_double),
                ("error", ctypes.c_double), ("variance", ctypes.c_double),
                ("tau", ctypes.c_double), ("R", ctypes.c_double),
                ("acceptance", ctypes.c_double)]


_P = ctypes.POINTER


class NqOpTable(ctypes.Structure):
    _fields_ = [("n_ops", ctypes.c_int32), ("n_rows", ctypes.c_int32),
                ("n_conns", ctypes.c_int32),
                ("op_n_sites", _P(ctypes.c_int32)), ("op_sites", _P(ctypes.c_int32)),
                ("op_row_offset", _P(ctypes.c_int32)), ("row_conn_offset", _P(ctypes.c_int32)),
                ("conn_mel", _P(ctypes.c_double)), ("conn_n_changes", _P(ctypes.c_int32)),
                ("conn_change_site", _P(ctypes.c_int32)),
                ("conn_change_value", _P(ctypes.c_int8))]


EXPORTS = {
    "nq_version": (ctypes.c_char_p, []),
    "nq_abi_version": (ctypes.c_int32, []),
    "nq_create": (ctypes.c_int, [_P(NqConfig), _P(ctypes.c_void_p)]),
    "nq_destroy": (None, [ctypes.c_void_p]),
    "nq_last_error": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    "nq_n_params": (ctypes.c_int64, [ctypes.c_void_p]),
    "nq_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32]),
    "nq_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32]),
    "nq_set_operator": (ctypes.c_int, [ctypes.c_void_p, _P(NqOpTable)]),
    "nq_set_exchange": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _P(ctypes.c_int32)]),
    "nq_set_rule_operator": (ctypes.c_int, [ctypes.c_void_p, _P(NqOpTable)]),
    "nq_set_symmetry": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _P(ctypes.c_int32)]),
    "nq_create_chain": (ctypes.c_int, [_P(NqConfig), ctypes.c_int32, _P(NqLayer), _P(ctypes.c_void_p)]),
    "nq_sample": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]),
    "nq_set_samples": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "nq_get_samples": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "nq_set_wait_limit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "nq_get_estimates": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "nq_logpsi": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "nq_logpsi_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                      ctypes.c_void_p, ctypes.c_void_p]),
    "nq_estimate": (ctypes.c_int, [ctypes.c_void_p, _P(NqMeasurement), ctypes.c_void_p,
                                   ctypes.c_void_p]),
    "nq_observable": (ctypes.c_int, [ctypes.c_void_p, _P(NqOpTable), _P(NqMeasurement), ctypes.c_void_p]),
    "nq_set_sr_tolerance": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double, ctypes.c_int32]),
    "nq_set_time_evolution": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "nq_sr_info": (ctypes.c_int, [ctypes.c_void_p, _P(ctypes.c_double)]),
    "nq_get_sr_matrix": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "nq_precondition": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                       ctypes.c_int32, ctypes.c_void_p]),
    "nq_update_descent": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "nq_vmc_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double,
                                   ctypes.c_double, _P(NqMeasurement)]),
    "nq_stage_times": (ctypes.c_int, [ctypes.c_void_p, _P(ctypes.c_float)]),
    "nq_kernel_launches": (ctypes.c_int64, [ctypes.c_void_p]),
    "nq_tuning": (ctypes.c_int, [ctypes.c_void_p, _P(ctypes.c_int32), ctypes.c_int32]),
    "nq_bench_steps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32,
                                      ctypes.c_double, ctypes.c_double, ctypes.c_int64,
                                      _P(ctypes.c_float)]),
    "nq_proposal_init": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, ctypes.c_uint64]),
    "nq_proposal_set_mix": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "nq_proposal_n_params": (ctypes.c_int64, [ctypes.c_void_p]),
    "nq_proposal_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "nq_proposal_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    "nq_proposal_logq": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "nq_proposal_sample": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "nq_proposal_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                        _P(ctypes.c_double)]),
    "nq_proposal_train": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                         _P(ctypes.c_double)]),
    "nq_proposal_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "nq_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, _P(ctypes.c_void_p)]),
    "nq_batch_destroy": (None, [ctypes.c_void_p]),
    "nq_batch_last_error": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    "nq_batch_size": (ctypes.c_int32, [ctypes.c_void_p]),
    "nq_batch_handle": (ctypes.c_void_p, [ctypes.c_void_p, ctypes.c_int32]),
    "nq_batch_vmc_step": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_void_p]),
    "nq_batch_bench_steps": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, ctypes.c_double,
                                            ctypes.c_double, _P(ctypes.c_float)]),
    "nq_batch_tuning": (ctypes.c_int, [ctypes.c_void_p, _P(ctypes.c_int32), ctypes.c_int32]),
    "nq_batch_kernel_launches": (ctypes.c_int64, [ctypes.c_void_p]),
    "nq_measurement_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                              ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p,
                                              ctypes.c_size_t]),
}

_lib = None
_lock = threading.Lock()


class NqError(RuntimeError):
    def __init__(self, status, message):
        self.status = status
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{name}: {message}")


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build(force=False, verbose=False):
    """Compile libnqcuda for sm_103a in-tree (parallel per translation unit)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    deps.append(os.path.join(INCLUDE, "nqcuda.h"))
    if not force and os.path.exists(LIB_PATH):
        t = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= t for d in deps):
            return LIB_PATH
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.basename(src).replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + ".tmp"
    cmd = [nvcc, "-shared", *ARCH, "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    """Load libnqcuda (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"libnqcuda is not built ({LIB_PATH} missing); "
                                   "run nqcuda.build() or __graft_entry__.build()")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in EXPORTS.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib
