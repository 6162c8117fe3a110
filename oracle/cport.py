"""Driver of the C restatement (oracle/cport.c) for one reference VMC
iteration, and its timing as the CPU baseline (test infrastructure, see
``oracle/__init__``).

Stages follow the reference: ``_sample_state!`` (C, OpenMP over chains),
``logψ_and_∇logψ!`` (C), the accumulator loop (C), centring and the force
(numpy), ``setup_algorithm!`` S = O_c O_c† via BLAS gemm (numpy/OpenBLAS,
as Julia's ``mul!`` in SRDirect.jl:32), ``precondition!`` Cholesky (scipy
LAPACK, as SRDirect.jl:79-81) and the Descent update.
"""
import os
import time

import numpy as np
import scipy.linalg as sla

from . import cbuild, exact, networks as nw
from .hilbert import Hilbert, SPIN


def flatten_ket_operator(H, N):
    """nq_op_table-style arrays from an oracle OpSum."""
    n_ops = len(H.ops)
    op_n_sites = np.zeros(n_ops, np.int32)
    op_sites = np.zeros(8 * n_ops, np.int32)
    op_row_offset = np.zeros(n_ops, np.int32)
    row_off, mel, nch, cs, cv = [0], [], [], [], []
    r0 = 0
    for o, op in enumerate(H.ops):
        op_n_sites[o] = len(op.sites)
        op_sites[8 * o:8 * o + len(op.sites)] = op.sites
        op_row_offset[o] = r0
        r0 += len(op.conns)
        for row in op.conns:
            for m, ch in row:
                mel += [m.real, m.imag]
                nch.append(len(ch))
                s8 = [0] * 8; v8 = [0] * 8
                for q, (s, v) in enumerate(ch):
                    s8[q], v8[q] = s, int(v)
                cs += s8; cv += v8
            row_off.append(len(nch))
    return [op_n_sites, op_sites, op_row_offset, np.array(row_off, np.int32),
            np.array(mel, np.float64), np.array(nch, np.int32), np.array(cs, np.int32),
            np.array(cv, np.int8)]


def _ptr(a):
    return a.ctypes.data


class PortRBM:
    """One reference VMC iteration in the C restatement.  ``precision`` "f64"
    runs complex128 throughout; "f32" runs the network, sampler and
    estimator in complex64 (the reference's default STD_REAL_PREC = Float32,
    src/NeuralQuantum.jl:57, with FP32 weights) and O, S, F and the Cholesky
    solve in complex64 as Julia would on ComplexF32 arrays."""

    def __init__(self, N, M, activation, hilb_kind, H, precision="f64"):
        self.N, self.M = N, M
        self.act = 0 if activation == nw.LOGCOSH else 1
        self.hilb = 0 if hilb_kind == SPIN else 1
        self.tab = flatten_ket_operator(H, N)
        self.L = cbuild.lib()
        self.precision = precision
        sfx = "_f32" if precision == "f32" else ""
        self.f_sample = getattr(self.L, "port_sample" + sfx)
        self.f_eval = getattr(self.L, "port_eval" + sfx)
        self.f_eloc = getattr(self.L, "port_eloc" + sfx)

    def iteration(self, params, B, L, burn, passes, seed, call, eps, lr, timings=None):
        N, M = self.N, self.M
        P = N + M + M * N
        params = np.ascontiguousarray(params, np.complex128)
        ns = B * L
        t0 = time.perf_counter()
        samples = np.empty((L, B, N), np.float64)
        self.f_sample(N, M, self.act, self.hilb, _ptr(params), B, L, burn, passes, seed, call, 0, _ptr(samples))
        t1 = time.perf_counter()
        flat = samples.reshape(ns, N)
        lp = np.empty(ns, np.complex128)
        O = np.empty((ns, P), np.complex128)
        self.f_eval(N, M, self.act, _ptr(params), ns, _ptr(flat), _ptr(lp), _ptr(O))
        E = np.empty(ns, np.complex128)
        self.f_eloc(N, M, self.act, self.hilb, _ptr(params), ns, _ptr(flat), _ptr(lp),
                    len(self.tab[0]), *[_ptr(a) for a in self.tab], _ptr(E))
        if self.precision == "f32":
            O = O.astype(np.complex64)
            E = E.astype(np.complex64)
        t2 = time.perf_counter()
        mean = O.mean(axis=0)
        O -= mean
        F = (E @ np.conj(O)) / ns
        S = np.conj(O.T @ np.conj(O)) / ns
        t3 = time.perf_counter()
        S[np.diag_indices_from(S)] += eps
        dw = sla.cho_solve(sla.cho_factor(S, lower=False, check_finite=False), F, check_finite=False)
        newp = params - lr * dw.astype(np.complex128)
        t4 = time.perf_counter()
        if timings is not None:
            timings.update(sample=t1 - t0, eval_eloc=t2 - t1, S=t3 - t2, solve=t4 - t3)
        return newp, samples, E, dw


def time_baseline(w, max_seconds=15.0, chains=None, quiet=False, precision="f32"):
    """Runs the reference iteration on a bounded number of chains and scales
    the chain-proportional stages to the full workload."""
    N, alpha = w["N"], w["alpha"]
    h = Hilbert(N, SPIN)
    H = exact.tfim_1d(h, w["h"], w["J"])
    port = PortRBM(N, alpha * N, nw.LOGCOSH, SPIN, H, precision=precision)
    net = nw.RBM(N, alpha * N, nw.LOGCOSH)
    nw.init_random_pars(net, np.random.default_rng(w["seed"]), sigma=1e-4)
    passes = w["passes"] + 1 if w["passes"] % 2 == 0 else w["passes"]
    full = w["chains"]
    B = chains or 16
    tm = {}
    # grow the sample until one iteration takes a noticeable share of the budget
    while True:
        port.iteration(net.flat(), B, w["chain_length"], w["burn"], passes, w["seed"], 0, w["eps"], w["lr"], tm)
        total = sum(tm.values())
        if chains or total > max_seconds / 4 or B >= full:
            break
        B = min(full, B * 4)
    scale = full / B
    per_step = (tm["sample"] + tm["eval_eloc"] + tm["S"]) * scale + tm["solve"]
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    return {"value": 1.0 / per_step, "unit": "SR steps/s", "cores": int(os.environ.get("OMP_NUM_THREADS", cores)),
            "kind": "port",
            "precision": precision,
            "sample": (f"{B} of {full} chains x {w['chain_length']} samples (C restatement of the reference "
                       f"path, {'FP32' if precision == 'f32' else 'FP64'} complex, OpenMP + OpenBLAS), "
                       f"chain-proportional stages scaled x{scale:g}"),
            "stage_s_measured": {k: round(v, 4) for k, v in tm.items()}}
