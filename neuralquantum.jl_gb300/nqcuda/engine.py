"""Thin object wrapper of one libnqcuda handle (include/nqcuda.h)."""
import ctypes

import numpy as np

from . import _lib
from .hilbert import SuperOpSpace, physical
from .networks import RBM, NDM, NDMSymm, RBMSplit, PureStateAnsatz, MixedStateAnsatz, Dense, DenseSplit, \
    PositiveDefR, WSum, af_logcosh, af_softplus


def make_config(net, hilb, n_chains, chain_length, burn, passes, seed, eval_precision=_lib.NQ_EVAL_F32,
                s_precision=_lib.NQ_S_F32, quirks=0, sampler_lanes=0, sr_algorithm=_lib.NQ_SR_DIRECT,
                sampler_kind=_lib.NQ_SAMPLER_METROPOLIS, rule=_lib.NQ_RULE_LOCAL,
                sampler_space=_lib.NQ_SPACE_NETWORK):
    """nq_config of one problem (include/nqcuda.h)."""
    cfg = _lib.NqConfig()
    ph = physical(hilb)
    if isinstance(net, RBM):
        cfg.network = _lib.NQ_NET_RBM
        cfg.n_hidden = net.M
        cfg.n_ancilla = 0
    elif isinstance(net, NDMSymm):
        cfg.network = _lib.NQ_NET_NDM_SYMM
        cfg.n_hidden = net.Mh
        cfg.n_ancilla = net.Ma
        cfg.n_symm = net.n_symm
    elif isinstance(net, NDM):
        cfg.network = _lib.NQ_NET_NDM
        cfg.n_hidden = net.Mh
        cfg.n_ancilla = net.Ma
    elif isinstance(net, MixedStateAnsatz):
        cfg.network = _lib.NQ_NET_MIXED_CHAIN
        cfg.n_hidden = net.chain.layers[0].n_out
        cfg.n_ancilla = 0
    elif isinstance(net, PureStateAnsatz):
        cfg.network = _lib.NQ_NET_CHAIN
        cfg.n_hidden = net.chain.layers[0].n_out
        cfg.n_ancilla = 0
    elif isinstance(net, RBMSplit):
        cfg.network = _lib.NQ_NET_RBM_SPLIT
        cfg.n_hidden = net.M
        cfg.n_ancilla = 0
    else:
        raise TypeError(f"unsupported network {type(net)}")
    f = getattr(net, "f", af_logcosh)
    cfg.activation = _lib.NQ_ACT_LOGCOSH if f == af_logcosh else _lib.NQ_ACT_SOFTPLUS
    cfg.hilbert = _lib.NQ_HILB_SPIN if ph.kind == "spin" else _lib.NQ_HILB_FOCK
    cfg.n_sites = ph.n_sites
    cfg.n_chains = n_chains
    cfg.chain_length = chain_length
    cfg.burn = burn
    cfg.passes = passes
    cfg.seed = seed
    cfg.eval_precision = eval_precision
    cfg.s_precision = s_precision
    cfg.quirks = quirks
    cfg.sampler_lanes = sampler_lanes
    cfg.sr_algorithm = sr_algorithm
    cfg.sampler_kind = sampler_kind
    cfg.rule = rule
    cfg.sampler_space = sampler_space
    return cfg


def chain_layers(net):
    """nq_layer array of a PureStateAnsatz's or MixedStateAnsatz's chain."""
    acts = {af_logcosh: _lib.NQ_ACT_LOGCOSH, af_softplus: _lib.NQ_ACT_SOFTPLUS, "identity": _lib.NQ_ACT_IDENTITY}
    layers = net.chain.layers
    arr = (_lib.NqLayer * len(layers))()
    width = net.N
    for k, l in enumerate(layers):
        if isinstance(l, DenseSplit):
            arr[k] = _lib.NqLayer(_lib.NQ_LAYER_DENSE_SPLIT, l.n_in, l.n_out, acts[l.f])
            width = l.n_out
        elif isinstance(l, PositiveDefR):
            arr[k] = _lib.NqLayer(_lib.NQ_LAYER_POSITIVE_DEF_R, l.n_in, l.n_out, acts[l.f])
            width = l.n_out
        elif isinstance(l, Dense):
            arr[k] = _lib.NqLayer(_lib.NQ_LAYER_DENSE, l.n_in, l.n_out, acts[l.f])
            width = l.n_out
        elif isinstance(l, WSum):
            arr[k] = _lib.NqLayer(_lib.NQ_LAYER_WSUM, l.n_in, 1, 0)
        else:
            arr[k] = _lib.NqLayer(_lib.NQ_LAYER_SUM, width, 1, 0)
    return arr


class Engine:
    def __init__(self, net, hilb, n_chains, chain_length, burn, passes, seed,
                 eval_precision=_lib.NQ_EVAL_F32, s_precision=_lib.NQ_S_F32, quirks=0,
                 sampler_lanes=0, sr_algorithm=_lib.NQ_SR_DIRECT, sampler_kind=_lib.NQ_SAMPLER_METROPOLIS,
                 rule=_lib.NQ_RULE_LOCAL, sampler_space=_lib.NQ_SPACE_NETWORK, _handle=None, _owner=None):
        L = _lib.lib()
        cfg = make_config(net, hilb, n_chains, chain_length, burn, passes, seed, eval_precision,
                          s_precision, quirks, sampler_lanes, sr_algorithm, sampler_kind, rule, sampler_space)
        self.complex_params = isinstance(net, (RBM, RBMSplit, PureStateAnsatz, MixedStateAnsatz))
        self.cfg = cfg
        self.lib = L
        self._owned = _handle is None
        self._owner = _owner                  # keeps a batch alive while its problem handles are used
        if _handle is None:
            self.h = ctypes.c_void_p()
            if isinstance(net, (PureStateAnsatz, MixedStateAnsatz)):
                st = L.nq_create_chain(ctypes.byref(cfg), len(net.chain.layers), chain_layers(net),
                                       ctypes.byref(self.h))
            else:
                st = L.nq_create(ctypes.byref(cfg), ctypes.byref(self.h))
            if st != _lib.NQ_OK:
                raise _lib.NqError(st, "nq_create failed (see stderr)")
            if isinstance(net, NDMSymm):
                perms = np.ascontiguousarray(net.permutations, dtype=np.int32)
                self._check(L.nq_set_symmetry(self.h, perms.shape[0],
                                              perms.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))
        else:
            self.h = ctypes.c_void_p(_handle)
        ph = physical(hilb)
        self.P = int(L.nq_n_params(self.h))
        self.N = ph.n_sites
        doubled = isinstance(hilb, SuperOpSpace) and sampler_space == _lib.NQ_SPACE_NETWORK
        self.nsites = 2 * ph.n_sites if doubled else ph.n_sites
        self.B, self.L = n_chains, chain_length
        self.passes = passes + 1 if passes % 2 == 0 else passes
        self._op = None

    def __del__(self):
        try:
            if self.h and self._owned:
                self.lib.nq_destroy(self.h)
                self.h = ctypes.c_void_p()
        except Exception:
            pass

    def _check(self, st):
        if st != _lib.NQ_OK:
            buf = ctypes.create_string_buffer(512)
            self.lib.nq_last_error(self.h, buf, 512)
            raise _lib.NqError(st, buf.value.decode(errors="replace"))

    # ---- parameters -------------------------------------------------------
    def set_params(self, flat):
        if self.complex_params:
            v = np.ascontiguousarray(flat, dtype=np.complex128)
            self._check(self.lib.nq_set_params(self.h, v.ctypes.data, self.P, _lib.NQ_DTYPE_C128))
        else:
            v = np.ascontiguousarray(np.real(flat), dtype=np.float64)
            self._check(self.lib.nq_set_params(self.h, v.ctypes.data, self.P, _lib.NQ_DTYPE_F64))

    def get_params(self):
        if self.complex_params:
            v = np.empty(self.P, np.complex128)
            self._check(self.lib.nq_get_params(self.h, v.ctypes.data, self.P, _lib.NQ_DTYPE_C128))
        else:
            v = np.empty(self.P, np.float64)
            self._check(self.lib.nq_get_params(self.h, v.ctypes.data, self.P, _lib.NQ_DTYPE_F64))
        return v

    def set_operator(self, table):
        self._op = table           # keep the arrays alive
        st = table.struct()
        self._check(self.lib.nq_set_operator(self.h, ctypes.byref(st)))

    def set_exchange(self, pairs):
        """Couplings of the exchange rule: (i, j) pairs of 0-based sites."""
        arr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        self._check(self.lib.nq_set_exchange(self.h, arr.shape[0],
                                             arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))))

    def set_rule_operator(self, table):
        """Move operator of the OperatorRule (an OpTable of ket sites)."""
        self._rule_op = table
        st = table.struct()
        self._check(self.lib.nq_set_rule_operator(self.h, ctypes.byref(st)))

    # ---- stages -------------------------------------------------------------
    def sample(self, call_index, want_samples=True, want_accept_bits=False):
        out = np.empty((self.L, self.B, self.nsites), np.int8) if want_samples else None
        steps = self.passes * (self.cfg.burn + self.L)
        bits = np.empty((steps, self.B), np.uint8) if want_accept_bits else None
        self._check(self.lib.nq_sample(self.h, call_index,
                                       out.ctypes.data if out is not None else None,
                                       bits.ctypes.data if bits is not None else None))
        return out, bits

    def set_samples(self, samples):
        v = np.ascontiguousarray(samples, dtype=np.int8)
        if v.size != self.L * self.B * self.nsites:
            raise ValueError("samples must hold L x B x nsites values")
        self._check(self.lib.nq_set_samples(self.h, v.ctypes.data))

    def get_samples(self):
        """The current sample buffer, (L, B, nsites) int8."""
        out = np.empty((self.L, self.B, self.nsites), np.int8)
        self._check(self.lib.nq_get_samples(self.h, out.ctypes.data))
        return out

    def get_estimates(self):
        """(local values (L, B), force F, update Δw) of the last estimate and
        solve on this handle, read back without recomputation."""
        loc = np.empty((self.L, self.B), np.complex128)
        dt = np.complex128 if self.complex_params else np.float64
        force = np.empty(self.P, dt)
        dw = np.empty(self.P, dt)
        self._check(self.lib.nq_get_estimates(self.h, loc.ctypes.data, force.ctypes.data, dw.ctypes.data))
        return loc, force, dw

    def logpsi(self, sigma, with_grad=False):
        """sigma: (n, nsites) site values -> logψ (n,) [, grad (n, P)]."""
        v = np.ascontiguousarray(sigma, dtype=np.int8)
        n = v.shape[0]
        out = np.empty(n, np.complex128)
        if with_grad:
            g = np.empty((n, self.P), np.complex128)
            self._check(self.lib.nq_logpsi_grad(self.h, v.ctypes.data, n, out.ctypes.data, g.ctypes.data))
            return out, g
        self._check(self.lib.nq_logpsi(self.h, v.ctypes.data, n, out.ctypes.data))
        return out

    def estimate(self, want_loc=False, want_force=False):
        m = _lib.NqMeasurement()
        loc = np.empty((self.L, self.B), np.complex128) if want_loc else None
        if want_force:
            force = np.empty(self.P, np.complex128 if self.complex_params else np.float64)
        else:
            force = None
        self._check(self.lib.nq_estimate(self.h, ctypes.byref(m),
                                         loc.ctypes.data if loc is not None else None,
                                         force.ctypes.data if force is not None else None))
        return m, loc, force

    def observable(self, table, want_loc=False):
        """Measurement of the local values of another operator on the current samples."""
        m = _lib.NqMeasurement()
        loc = np.empty((self.L, self.B), np.complex128) if want_loc else None
        st = table.struct()
        self._check(self.lib.nq_observable(self.h, ctypes.byref(st), ctypes.byref(m),
                                           loc.ctypes.data if loc is not None else None))
        return m, loc

    def set_sr_tolerance(self, tol, maxiter):
        self._check(self.lib.nq_set_sr_tolerance(self.h, float(tol), int(maxiter)))

    def set_time_evolution(self, on):
        """SR(time_evo=...): the solves take i F instead of F."""
        self._check(self.lib.nq_set_time_evolution(self.h, 1 if on else 0))

    def set_wait_limit(self, ns):
        """Limit of every grid-barrier wait of the solve kernels (0 = 1 s)."""
        self._check(self.lib.nq_set_wait_limit(self.h, int(ns)))

    def sr_info(self):
        """[iterations, |r|/|F|] of the last matrix-free SR solve, or
        [FP64-residual corrections, last |Δx|/|x|] of the last direct solve."""
        v = (ctypes.c_double * 2)()
        self._check(self.lib.nq_sr_info(self.h, v))
        return int(v[0]), float(v[1])

    def sr_matrix(self):
        S = np.empty((self.P, self.P), np.complex128 if self.complex_params else np.float64, order="F")
        self._check(self.lib.nq_get_sr_matrix(self.h, S.ctypes.data))
        return S

    def precondition(self, kind=0, eps=0.001, lam0=100.0, b=0.95, lam_min=1e-4, it=1):
        dw = np.empty(self.P, np.complex128 if self.complex_params else np.float64)
        self._check(self.lib.nq_precondition(self.h, kind, eps, lam0, b, lam_min, it, dw.ctypes.data))
        return dw

    def update_descent(self, lr):
        self._check(self.lib.nq_update_descent(self.h, lr))

    def vmc_step(self, call_index, eps, lr):
        m = _lib.NqMeasurement()
        self._check(self.lib.nq_vmc_step(self.h, call_index, eps, lr, ctypes.byref(m)))
        return m

    def stage_times(self):
        """[sample, eval, force+stats, S, solve, update, sampler kernel, S kernel,
        inversion, rhs, first solve, refinement] ms."""
        a = (ctypes.c_float * 12)()
        self._check(self.lib.nq_stage_times(self.h, a))
        return list(a)

    def bench_steps(self, call0, n, eps, lr, flush_bytes):
        a = (ctypes.c_float * n)()
        self._check(self.lib.nq_bench_steps(self.h, call0, n, eps, lr, flush_bytes, a))
        return list(a)

    def tuning(self):
        """Autotuned choices: lanes per chain and threads per block of the
        sampler, split-K of the S accumulation."""
        a = (ctypes.c_int32 * 3)()
        self._check(self.lib.nq_tuning(self.h, a, 3))
        return {"sampler_lanes": a[0], "gram_ksplit": a[1], "sampler_block": a[2]}

    def kernel_launches(self):
        return int(self.lib.nq_kernel_launches(self.h))

    # ---- learned autoregressive proposal (MADE), nq_proposal_* -------------
    def proposal_init(self, hidden=128, p_ar=0.5, seed=0):
        self._check(self.lib.nq_proposal_init(self.h, hidden, float(p_ar), seed))
        self.proposal_P = int(self.lib.nq_proposal_n_params(self.h))

    def proposal_set_mix(self, p_ar):
        self._check(self.lib.nq_proposal_set_mix(self.h, float(p_ar)))

    def proposal_set_params(self, flat):
        v = np.ascontiguousarray(flat, dtype=np.float32)
        self._check(self.lib.nq_proposal_set_params(self.h, v.ctypes.data, v.size))

    def proposal_get_params(self):
        v = np.empty(self.proposal_P, dtype=np.float32)
        self._check(self.lib.nq_proposal_get_params(self.h, v.ctypes.data, v.size))
        return v

    def proposal_logq(self, x_bits):
        x = np.ascontiguousarray(x_bits, dtype=np.uint64)
        out = np.empty(x.size, dtype=np.float32)
        self._check(self.lib.nq_proposal_logq(self.h, x.ctypes.data, x.size, out.ctypes.data))
        return out

    def proposal_sample(self, call_index, slots):
        x = np.empty(self.B * slots, dtype=np.uint64)
        lq = np.empty(self.B * slots, dtype=np.float32)
        self._check(self.lib.nq_proposal_sample(self.h, call_index, slots, x.ctypes.data, lq.ctypes.data))
        return x.reshape(self.B, slots), lq.reshape(self.B, slots)

    def proposal_grad(self, x_bits):
        x = np.ascontiguousarray(x_bits, dtype=np.uint64)
        g = np.empty(self.proposal_P, dtype=np.float32)
        nll = ctypes.c_double()
        self._check(self.lib.nq_proposal_grad(self.h, x.ctypes.data, x.size, g.ctypes.data, ctypes.byref(nll)))
        return g, nll.value

    def proposal_train(self, steps, batch, lr):
        nll = ctypes.c_double()
        self._check(self.lib.nq_proposal_train(self.h, steps, batch, float(lr), ctypes.byref(nll)))
        return nll.value

    def proposal_stats(self):
        v = np.zeros(2, dtype=np.uint64)
        self._check(self.lib.nq_proposal_stats(self.h, v.ctypes.data))
        return int(v[0]), int(v[1])


class ProblemBatch:
    """Many independent RBM problems stepped together (nq_batch_*): one
    sampler launch, one estimator launch and one inversion launch for all of
    them per SR step, inside one CUDA graph.  ``problems`` is a list of
    (net, hilb, operator) with RBM networks of one activation; every problem
    gets n_chains chains of chain_length samples."""

    def __init__(self, problems, n_chains, chain_length, burn, passes=None, seed=0x4E51,
                 s_precision=_lib.NQ_S_TF32):
        from .operators import op_table
        L = _lib.lib()
        self.lib = L
        n = len(problems)
        cfgs = (_lib.NqConfig * n)()
        for i, (net, hilb, _) in enumerate(problems):
            ps = passes if passes is not None else physical(hilb).n_sites
            cfgs[i] = make_config(net, hilb, n_chains, chain_length, burn, ps, seed + 7919 * i,
                                  _lib.NQ_EVAL_F32, s_precision)
        self.b = ctypes.c_void_p()
        st = L.nq_batch_create(ctypes.cast(cfgs, ctypes.c_void_p), n, ctypes.byref(self.b))
        if st != _lib.NQ_OK:
            raise _lib.NqError(st, "nq_batch_create failed")
        self.engines = []
        for i, (net, hilb, op) in enumerate(problems):
            ps = passes if passes is not None else physical(hilb).n_sites
            h = L.nq_batch_handle(self.b, i)
            e = Engine(net, hilb, n_chains, chain_length, burn, ps, seed + 7919 * i, _lib.NQ_EVAL_F32,
                       s_precision, _handle=h, _owner=self)
            e.set_params(net.flat())
            e.set_operator(op_table(op))
            self.engines.append(e)
        self.n = n

    def _check(self, st):
        if st != _lib.NQ_OK:
            buf = ctypes.create_string_buffer(512)
            self.lib.nq_batch_last_error(self.b, buf, 512)
            raise _lib.NqError(st, buf.value.decode(errors="replace"))

    def vmc_step(self, call_index, eps, lr):
        ms = (_lib.NqMeasurement * self.n)()
        self._check(self.lib.nq_batch_vmc_step(self.b, call_index, eps, lr, ctypes.cast(ms, ctypes.c_void_p)))
        return list(ms)

    def bench_steps(self, call0, n, eps, lr):
        out = np.zeros(n, np.float32)
        self._check(self.lib.nq_batch_bench_steps(self.b, call0, n, eps, lr,
                                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_float))))
        return out

    def tuning(self):
        v = (ctypes.c_int32 * 4)()
        self._check(self.lib.nq_batch_tuning(self.b, v, 4))
        return {"sampler_lanes": v[0], "estimator_threads": v[1], "inversion_ctas": v[2],
                "kernels_per_step": v[3]}

    def kernel_launches(self):
        return int(self.lib.nq_batch_kernel_launches(self.b))

    def __del__(self):
        try:
            for e in getattr(self, "engines", []):
                e.h = ctypes.c_void_p()
            if getattr(self, "b", None):
                self.lib.nq_batch_destroy(self.b)
                self.b = ctypes.c_void_p()
        except Exception:
            pass
