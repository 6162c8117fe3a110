"""nq_measurement_noalloc: the chain statistics of nq_estimate on
caller-owned device values, with its scratch in a fixed device array.

It is compared with the handle path (nq_estimate) on the same local
energies, on two calls in a row (the second call reuses the scratch the
first one left behind), and with the oracle for the squared-modulus kind.
Tolerance: relative 1e-12 (both paths run the same FP64 reductions on the
same FP32 inputs).  The device buffers of the test itself come from torch;
the entry point allocates nothing.
"""
import ctypes

import numpy as np
import pytest

import nqcuda as nq
from oracle import stats as ost

pytestmark = pytest.mark.gpu


def _engine(B=256, L=12, N=8):
    hilb = nq.HomogeneousSpin(N)
    net = nq.RBM(np.complex64, N, 2, nq.af_logcosh)
    nq.init_random_pars_(net, sigma=0.05, rng=np.random.default_rng(3))
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H = H - nq.sigmax(hilb, i)
        H = H + nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    s = nq.MetropolisSampler(nq.LocalRule(), L, N, burn=5, seed=77)
    return nq.BatchedSampler(net, s, H, nq.SR(eps=0.01), batch_sz=B).engine


def _call(lib, vals, dtype, B, L, kind, out, stream):
    err = ctypes.create_string_buffer(256)
    st = lib.nq_measurement_noalloc(vals, dtype, B, L, kind, out, stream, err, 256)
    return st, err.value.decode()


def test_noalloc_measurement_matches_estimate(nqlib):
    torch = pytest.importorskip("torch")
    lib = nq._lib.lib()
    eng = _engine()
    eng.sample(0, want_samples=False)
    m, loc, _ = eng.estimate(want_loc=True)
    ref = np.array([m.mean_re, m.mean_im, m.error, m.variance, m.tau, m.R])
    stream = torch.cuda.current_stream().cuda_stream
    for dtype, cdt in ((nq._lib.NQ_DTYPE_C64, torch.complex64), (nq._lib.NQ_DTYPE_C128, torch.complex128)):
        vals = torch.from_numpy(loc.reshape(-1).copy()).to(cdt).cuda()      # [L][B], chain fastest
        out = torch.empty(6, dtype=torch.float64, device="cuda")
        for _ in range(2):
            out.fill_(float("nan"))
            st, msg = _call(lib, vals.data_ptr(), dtype, eng.B, eng.L, 0, out.data_ptr(), stream)
            assert st == nq._lib.NQ_OK, msg
            torch.cuda.synchronize()
            np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-12, atol=1e-14)


def test_noalloc_squared_modulus_and_limits(nqlib):
    torch = pytest.importorskip("torch")
    lib = nq._lib.lib()
    rng = np.random.default_rng(9)
    B, L = 1000, 7
    v = (rng.standard_normal((L, B)) + 1j * rng.standard_normal((L, B))).astype(np.complex64)
    vals = torch.from_numpy(v.reshape(-1).copy()).cuda()
    out = torch.empty(6, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    o = ost.stat_analysis((np.abs(v.astype(np.complex128)) ** 2).T)
    want = np.array([o["mean"], 0.0, o["error"], o["variance"], o["tau"], o["R"]])
    for _ in range(2):
        st, msg = _call(lib, vals.data_ptr(), nq._lib.NQ_DTYPE_C64, B, L, 1, out.data_ptr(), stream)
        assert st == nq._lib.NQ_OK, msg
        torch.cuda.synchronize()
        np.testing.assert_allclose(out.cpu().numpy(), want, rtol=1e-10, atol=1e-14)
    # sizes beyond the fixed scratch are refused before anything is launched
    st, msg = _call(lib, vals.data_ptr(), nq._lib.NQ_DTYPE_C64, 65537, 1, 0, out.data_ptr(), stream)
    assert st == nq._lib.NQ_ERR_ARG and "65536" in msg
    # host memory is refused
    host = np.zeros(16, np.complex64)
    st, msg = _call(lib, host.ctypes.data, nq._lib.NQ_DTYPE_C64, 4, 4, 0, out.data_ptr(), stream)
    assert st == nq._lib.NQ_ERR_ARG and "device" in msg
