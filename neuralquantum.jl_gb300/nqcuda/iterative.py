"""The reference's user loop on top of libnqcuda.

    is = BatchedSampler(net, sampler, H, SR(ϵ=0.01); batch_sz=4096)
    for i in range(1, 301):
        ldata, prec = sample_(is)            # sample!(is)
        grad = precondition_(prec, algo, i)  # precondition!(prec, algo, i)
        update_(Descent(0.01), net, grad)    # Optimisers.update!(opt, net, grad)

Reference: src/IterativeInterface/build_Batched.jl:1-14 (BatchedSampler),
Samplers/CostFun/BatchedValSampler.jl:117-139 and BatchedGradSampler.jl:77-123
(sample!), src/Algorithms/SR/SR.jl:50-57 and SRDirect.jl:51-90
(SR / precondition!), src/Optimisers/rules.jl:11-17 and apply.jl:25-32
(Descent / update!).
"""
import numpy as np

from . import _lib
from .engine import Engine
from .operators import KLocalLiouvillian, op_table
from .hilbert import SuperOpSpace
from .stats import Measurement

sr_shift, sr_multiplicative, sr_none = 0, 1, 2
sr_cholesky, sr_cg, sr_minres, sr_qlp, sr_lsq = "sr_cholesky", "sr_cg", "sr_minres", "sr_qlp", "sr_lsq"
sr_diag, sr_div, sr_pivcholesky = "sr_diag", "sr_div", "sr_pivcholesky"
_ITERATIVE = (sr_cg, sr_minres, sr_qlp, sr_lsq)
_DIRECT = (sr_cholesky, sr_diag, sr_div)


class SR:
    """``SR(T; ϵ=0.001, precision=1e-4, precondition_type=sr_shift,
    algorithm=sr_cholesky, λ0=100, b=0.95, λmin=1e-4, time_evo=false)``
    (SR.jl:41-57).  ``time_evo`` solves with i F instead of F
    (SRDirect.jl:27, SRIterative.jl:33), Re(i F) for real parameters.
    sr_cholesky, sr_diag (pinv) and sr_div form S and solve the preconditioned
    system directly (the shifted S is positive definite, where the three
    agree; a singular S with sr_none is refused, not pseudo-inverted); the
    iterative algorithms run the engine's matrix-free conjugate-gradient
    solve of the same shifted system to the relative residual ``precision``.
    sr_pivcholesky is not implemented by the reference's precondition!
    either (SRDirect.jl:84-86)."""

    def __init__(self, eps=0.001, precondition_type=sr_shift, algorithm=sr_cholesky,
                 lam0=100.0, b=0.95, lam_min=1e-4, precision=1e-4, time_evo=False):
        if algorithm not in _DIRECT and algorithm not in _ITERATIVE:
            raise NotImplementedError(f"unknown SR algorithm {algorithm}")
        self.time_evo = bool(time_evo)
        self.eps, self.precondition_type = float(eps), precondition_type
        self.lam0, self.b, self.lam_min = float(lam0), float(b), float(lam_min)
        self.algorithm, self.precision = algorithm, float(precision)

    @property
    def iterative(self):
        return self.algorithm in _ITERATIVE


class Descent:
    def __init__(self, eta):
        self.eta = float(eta)


class SRCache:
    """What ``sample!`` returns as the preconditioner cache: S and F live on
    the device inside the engine."""

    def __init__(self, sampler):
        self.sampler = sampler


class Gradient:
    """Δw returned by ``precondition_``; the values also stay on the device."""

    def __init__(self, sampler, values):
        self.sampler = sampler
        self.values = values


class BatchedSampler:
    def __init__(self, net, sampler, prob, algo=None, batch_sz=16, eval_precision=_lib.NQ_EVAL_F32,
                 s_precision=_lib.NQ_S_F32, reference_quirks=False):
        self.net = net
        self.sampler = sampler
        self.prob = prob
        self.algo = algo if algo is not None else SR()
        self.liouvillian = isinstance(prob, KLocalLiouvillian)
        hilb = prob.hilb if not self.liouvillian else prob.hilb
        quirks = _lib.NQ_QUIRK_STALE_LAST_SLOT if reference_quirks else 0
        self.reference_quirks = bool(reference_quirks)
        sr_alg = _lib.NQ_SR_CG if self.algo.iterative else _lib.NQ_SR_DIRECT
        exch = getattr(getattr(sampler, "rule", None), "couplings", None)
        move_op = getattr(getattr(sampler, "rule", None), "operator", None)
        rule = _lib.NQ_RULE_LOCAL
        if exch is not None:
            rule = _lib.NQ_RULE_EXCHANGE
        elif move_op is not None:
            rule = _lib.NQ_RULE_OPERATOR
        self.engine = Engine(net, hilb, batch_sz, sampler.chain_length, sampler.burn_length,
                             sampler.passes, sampler.seed, eval_precision, s_precision, quirks,
                             sr_algorithm=sr_alg, sampler_kind=getattr(sampler, "kind", 0), rule=rule)
        if exch is not None:
            self.engine.set_exchange(exch)
        if move_op is not None:
            self.engine.set_rule_operator(op_table(move_op))
        if self.algo.iterative:
            self.engine.set_sr_tolerance(self.algo.precision, 10 * self.engine.P)
        if getattr(self.algo, "time_evo", False):
            self.engine.set_time_evolution(True)
        self.engine.set_params(net.flat())
        self.engine.set_operator(op_table(prob))
        self.calls = 0
        self.last_samples = None

    def sample_(self, keep_samples=False):
        out, _ = self.engine.sample(self.calls, want_samples=keep_samples)
        self.calls += 1
        if keep_samples:
            self.last_samples = out
        m, _, _ = self.engine.estimate()
        mean = complex(m.mean_re, m.mean_im) if not self.liouvillian else m.mean_re
        return Measurement(mean, m.error, m.variance, m.tau, m.R), SRCache(self)

    def step(self, lr, eps=None):
        """One whole iteration (sample!, precondition! with sr_shift, update!)
        replayed from a captured CUDA graph."""
        eps = self.algo.eps if eps is None else eps
        m = self.engine.vmc_step(self.calls, eps, lr)
        self.calls += 1
        mean = complex(m.mean_re, m.mean_im) if not self.liouvillian else m.mean_re
        return Measurement(mean, m.error, m.variance, m.tau, m.R)

    def sync_net(self):
        self.net.set_flat(self.engine.get_params())
        return self.net


def sample_(is_):
    return is_.sample_()


def precondition_(prec, algo, it):
    """``precondition!(prec, SR, it)``.  With reference_quirks the reference's
    handling of sr_multiplicative is reproduced: sr_cholesky and sr_div solve
    with S itself and the multiplicative shift reaches only sr_diag
    (SRDirect.jl:64-83)."""
    eng = prec.sampler.engine
    kind = algo.precondition_type
    if getattr(prec.sampler, "reference_quirks", False) and kind == sr_multiplicative and \
            algo.algorithm in (sr_cholesky, sr_div):
        kind = sr_none
    dw = eng.precondition(kind, algo.eps, algo.lam0, algo.b, algo.lam_min, it)
    return Gradient(prec.sampler, dw)


def update_(opt, net, grad):
    s = grad.sampler
    if s.net is not net:
        raise ValueError("the gradient belongs to another network")
    s.engine.update_descent(opt.eta)
    s.sync_net()
    return net


class BatchedObsKetSampler:
    """``BatchedObsKetSampler`` (Obs/BatchedObsKetSampler.jl:1-60): local
    values of named observables on the samples of the last sample call of a
    ``BatchedSampler``, with their ``Measurement``."""

    def __init__(self, sampler):
        self.sampler = sampler
        self.observables = {}
        self.results = {}

    def add_observable_(self, name, op):
        self.observables[name] = op_table(op)

    def compute_observable(self, table):
        m, _ = self.sampler.engine.observable(table)
        return Measurement(complex(m.mean_re, m.mean_im), m.error, m.variance, m.tau, m.R)

    def compute_observables(self):
        for name, table in self.observables.items():
            self.results[name] = self.compute_observable(table)
        return self.results


class BatchedObsDMSampler:
    """``BatchedObsDMSampler(net, sampler, hilb_doubled; batch_sz)``
    (Obs/BatchedObsDMSampler.jl:24-105): its own chains on the physical
    space with p(σ) ∝ ρ(σ,σ), and for each observable Ô the local values
    O_loc(σ) = Σ_σ' O_σσ' ρ(σ',σ)/ρ(σ,σ), whose mean is Tr(ρÔ)/Tr(ρ).  Every
    compute call draws a new set of samples (sample call index 0, 1, ...);
    the network's current parameters are uploaded first."""

    def __init__(self, net, sampler, hilb_doubled, batch_sz=16, eval_precision=_lib.NQ_EVAL_F32,
                 reference_quirks=False):
        from .networks import NDM, RBMSplit
        if not isinstance(net, (NDM, RBMSplit)):             # NDMSymm is an NDM
            raise TypeError("BatchedObsDMSampler needs a density-matrix network (NDM, RBMSplit)")
        self.net = net
        self.sampler = sampler
        self.hilb = hilb_doubled
        quirks = _lib.NQ_QUIRK_STALE_LAST_SLOT if reference_quirks else 0
        rule = getattr(sampler, "rule", None)
        if getattr(rule, "couplings", None) is not None or getattr(rule, "operator", None) is not None:
            raise NotImplementedError("the diagonal sampler uses LocalRule")
        self.engine = Engine(net, hilb_doubled, batch_sz, sampler.chain_length, sampler.burn_length,
                             sampler.passes, sampler.seed, eval_precision, _lib.NQ_S_F32, quirks,
                             sampler_kind=getattr(sampler, "kind", 0), sampler_space=_lib.NQ_SPACE_DIAGONAL)
        self.engine.set_params(net.flat())
        self.observables = {}
        self.results = {}
        self.calls = 0

    def add_observable_(self, name, op):
        self.observables[name] = op_table(op)

    def _sample(self):
        self.engine.set_params(self.net.flat())
        self.engine.sample(self.calls, want_samples=False)
        self.calls += 1

    def _eval(self, table):
        m, _ = self.engine.observable(table)
        return Measurement(complex(m.mean_re, m.mean_im), m.error, m.variance, m.tau, m.R)

    def compute_observable(self, op):
        self._sample()
        return self._eval(op if hasattr(op, "struct") else op_table(op))

    def compute_observables(self):
        if not self.observables:
            return None
        self._sample()
        for name, table in self.observables.items():
            self.results[name] = self._eval(table)
        return self.results


def compute_observables(obs):
    return obs.compute_observables()


def add_observable_(obs, name, op):
    obs.add_observable_(name, op)
