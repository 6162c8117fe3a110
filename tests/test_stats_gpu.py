"""Measurement statistics on the GPU (stats.jl:26-50) at a large offset and
a tiny spread: local values of -40 + 1e-6 noise, where the spread of the
chain means is 1e-12 of the squared mean.  The chain-statistics kernels centre
every 64-chain block on its own mean and merge blocks pairwise, so error, tau
and R keep their digits; the values reach the kernels through the statistics
entry point that reads caller-owned device memory.
Tolerance: relative 1e-6 on error, variance, tau, R; 1e-12 on the mean."""
import ctypes

import numpy as np
import pytest

import nqcuda as nq
from oracle import stats as ost

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("B,L", [(1000, 9), (64, 20), (4096, 5), (7, 3)])
def test_statistics_large_offset_small_spread(nqlib, B, L):
    torch = pytest.importorskip("torch")
    lib = nq._lib.lib()
    rng = np.random.default_rng(B + L)
    v = -40.0 + 1e-6 * (rng.standard_normal((L, B)) + 1j * rng.standard_normal((L, B)))
    vals = torch.from_numpy(v.reshape(-1).copy()).cuda()
    out = torch.empty(6, dtype=torch.float64, device="cuda")
    err = ctypes.create_string_buffer(256)
    st = lib.nq_measurement_noalloc(vals.data_ptr(), nq._lib.NQ_DTYPE_C128, B, L, 0, out.data_ptr(),
                                    torch.cuda.current_stream().cuda_stream, err, 256)
    assert st == nq._lib.NQ_OK, err.value
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    o = ost.stat_analysis(v.T)
    assert abs(complex(got[0], got[1]) - o["mean"]) < 1e-12 * 40
    for k, name in ((2, "error"), (3, "variance"), (4, "tau"), (5, "R")):
        ref = o[name]
        assert abs(got[k] - ref) <= 1e-6 * max(abs(ref), 1e-300) + (1e-9 if name == "tau" else 0.0), (name, got[k], ref)
