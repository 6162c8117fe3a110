"""Benchmark of one VMC iteration (sample! + precondition! + update!) on
the workload of the transverse-field Ising chain:

  N = 20 spins, periodic, H = -h Σσx + J Σσzσz with h = J = 1; complex RBM
  α = 2 (40 hidden units, FP32 weights, logcosh activation, spin ±1),
  4096 Metropolis chains, 20 samples per chain, 50 burn sweeps, passes =
  N -> 21 local flips per sweep, each sample enumerates N + 1 connected
  elements; SR with diagonal shift 0.01 (Cholesky), Descent lr 0.01.

One step = one SR iteration on the device, replayed from a CUDA graph.
`value` is SR steps/s of the whole job; `e2e` is the same metric measured
through the public API with the parameters uploaded from and downloaded to
host memory every step.  `--impl reference` times the CPU restatement of the
reference algorithm (the oracle port) on the host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "neuralquantum.jl_gb300"))

import numpy as np  # noqa: E402

WORKLOAD = dict(N=20, alpha=2, h=1.0, J=1.0, chains=4096, chain_length=20, burn=50, passes=20,
                eps=0.01, lr=0.01, seed=0x4E51)
METRIC = "SR steps/s (N=20 TFIM, complex RBM α=2, 4096 chains x 20 samples)"
L2_FLUSH_BYTES = 256 << 20


def workload_config(extra=None):
    w = WORKLOAD
    cfg = {"workload": "tfim1d_N20_rbm_alpha2_4096x20", "n_sites": w["N"], "hidden": w["alpha"] * w["N"],
           "chains": w["chains"], "samples_per_chain": w["chain_length"], "burn_sweeps": w["burn"],
           "passes": w["passes"] + 1, "sr_shift": w["eps"], "lr": w["lr"],
           "l2": "flushed between timed steps (256 MiB device write)"}
    if extra:
        cfg.update(extra)
    return cfg


# --------------------------------------------------------------------------
# clocks sampling during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.lines = []
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# --------------------------------------------------------------------------
# GB300 arm
# --------------------------------------------------------------------------
def build_sampler(s_precision=None):
    import nqcuda as nq
    w = WORKLOAD
    hilb = nq.HomogeneousSpin(w["N"])
    H = nq.LocalOperator(hilb)
    for i in range(1, w["N"] + 1):
        H = H - w["h"] * nq.sigmax(hilb, i)
        H = H + w["J"] * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % w["N"] + 1)
    net = nq.RBM(np.complex64, w["N"], w["alpha"], nq.af_logcosh)
    nq.init_random_pars_(net, sigma=1e-4, rng=np.random.default_rng(w["seed"]))
    smp = nq.MetropolisSampler(nq.LocalRule(), w["chain_length"], w["passes"], burn=w["burn"],
                               seed=w["seed"])
    sp = nq._lib.NQ_S_TF32 if s_precision is None else s_precision
    is_ = nq.BatchedSampler(net, smp, H, nq.SR(eps=w["eps"]), batch_sz=w["chains"], s_precision=sp,
                            eval_precision=eval_precision_choice())
    return nq, net, is_


def eval_precision_choice():
    """Evaluation precision of the bench workload: FP32 on CUDA cores unless
    NQ_BENCH_EVAL_PRECISION names another nq_eval_precision (for example
    NQ_EVAL_TC_BF16X2, θ on tcgen05, for a profile of that kernel)."""
    import nqcuda as nq
    env = os.environ.get("NQ_BENCH_EVAL_PRECISION")
    return getattr(nq._lib, env) if env else nq._lib.NQ_EVAL_F32


def s_precision_choice():
    import nqcuda as nq
    env = os.environ.get("NQ_BENCH_S_PRECISION")
    if env:
        return getattr(nq._lib, env)
    return nq._lib.NQ_S_TF32


# DRAM bytes (read + write) of one gram_tf32_kernel launch on this workload, from
# the ncu capture summarised in profiles/gram_tf32_c1.txt
GRAM_TRAFFIC_BYTES = 701.59e6
# one ncu capture of a production launch of the Metropolis kernel on this
# workload (profiles/rbm_sampler_c1.txt): warp instructions
# (smsp__inst_executed.sum), the capture's duration, its issue-active share and
# the acceptance of that launch (the accepted-flip update is most of the
# difference between launches)
SAMPLER_NCU = {"warp_instructions": 534.2e6, "duration_us": 726.0, "issue_active_pct": 65.7, "acceptance": 0.888,
               "warp_instructions_per_warp_step": 177.4}
# DRAM bytes (read + write) of one sampler launch (same capture)
SAMPLER_TRAFFIC_BYTES = 62e3
# algorithmic FP32 flops of one Metropolis proposal per hidden unit: the ratio
# t0 + g t1 (complex FMA, 8), |r|^2 (3) and the running product (1); and per
# hidden unit of an accepted flip: θ += W dv (4), num = g + τ (2),
# den = 1 + g τ (8), |den|^2 (3), 1/|den|^2 (1), num conj(den) (6), scaling (2)
SAMPLER_FLOPS_RATIO = 12
SAMPLER_FLOPS_ACCEPT = 26


def effective_samples_per_s(loc, sample_ms):
    from nqcuda.stats import integrated_autocorr_time
    tau = integrated_autocorr_time(loc.T)
    ns = loc.size
    return ns / tau / (sample_ms / 1e3), tau


def run_gb300(args, barrier=None):
    import nqcuda as nq
    nq.build()
    peaks = {}
    pk = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    sp = s_precision_choice()
    nq_, net, is_ = build_sampler(sp)
    eng = is_.engine
    w = WORKLOAD
    # warm-up (also captures the graph)
    for i in range(args.warmup):
        eng.vmc_step(i, w["eps"], w["lr"])
    launches0 = eng.kernel_launches()
    if barrier:
        barrier()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms = eng.bench_steps(args.warmup, args.steps, w["eps"], w["lr"], L2_FLUSH_BYTES)   # synchronises
    if barrier:
        barrier()
    launches = eng.kernel_launches() - launches0
    total_ms = float(np.sum(ms))
    ms_step = total_ms / args.steps
    value = 1e3 / ms_step

    # the same step with S accumulated from BF16 O (tcgen05 kind::f16)
    modes = {}
    if sp != nq._lib.NQ_S_BF16:
        _, _, is_bf = build_sampler(nq._lib.NQ_S_BF16)
        e_bf = is_bf.engine
        for i in range(args.warmup):
            e_bf.vmc_step(i, w["eps"], w["lr"])
        ms_bf = float(np.mean(e_bf.bench_steps(args.warmup, max(10, args.steps // 4), w["eps"], w["lr"],
                                               L2_FLUSH_BYTES)))
        modes["bf16_S"] = {"ms_per_step": ms_bf, "sr_steps_per_s": 1e3 / ms_bf,
                           "S_accumulation_ms": None, "note": "S from BF16 O, FP32 accumulation; S within 1e-2 "
                                                             "relative of the FP64 oracle (tests/test_tc_gpu.py)"}
        e_bf.sample(10 ** 6, want_samples=False)
        e_bf.estimate()
        modes["bf16_S"]["S_accumulation_ms"] = float(e_bf.stage_times()[7])
        del e_bf, is_bf

    # staged pass: per-stage and per-kernel device times, E_loc for ESS
    call = args.warmup + args.steps + 10
    eng.sample(call, want_samples=False)
    m, loc, _ = eng.estimate(want_loc=True)
    eng.precondition(0, w["eps"])
    eng.update_descent(w["lr"])
    st = eng.stage_times()
    ess, tau = effective_samples_per_s(loc, st[0])

    # e2e through the public API with host parameters every step
    flat = net.flat()
    t0 = time.perf_counter()
    for i in range(args.steps):
        eng.set_params(flat)
        eng.vmc_step(call + 1 + i, w["eps"], w["lr"])
        flat = eng.get_params()
    e2e_s = time.perf_counter() - t0
    P = eng.P
    e2e = {"value": args.steps / e2e_s, "unit": "SR steps/s", "h2d_bytes_per_step": 16 * P,
           "d2h_bytes_per_step": 16 * P + 8 * 7}

    # roofline: the dominant kernel (the Metropolis sampler, FP32 CUDA cores)
    # with its algorithmic flops; the tensor-core S accumulation as a second entry
    Ns = w["chains"] * w["chain_length"]
    kernels = {"sampler": st[6], "S_accumulation": st[7], "inversion": st[8]}
    ksum = sum(kernels.values())
    stages = {"sample": st[0], "eval_estimator": st[1], "force_stats": st[2], "S": st[3],
              "solve": st[4], "update": st[5]}
    clk_sum = clk.summary()
    sm_ghz = (clk_sum.get("sm_mhz") or 2070.0) / 1000.0
    M = w["alpha"] * w["N"]
    proposals = w["chains"] * (w["passes"] + 1) * (w["burn"] + w["chain_length"])
    flops_per_proposal = SAMPLER_FLOPS_RATIO * M + m.acceptance * SAMPLER_FLOPS_ACCEPT * M
    fp32_peak = 152 * 128 * 2 * sm_ghz * 1e9 / 1e12
    samp_tflops = proposals * flops_per_proposal / (st[6] * 1e-3) / 1e12
    roof = {"kernel": "rbm_sampler_kernel (Metropolis, θ-cache)", "bound": "fp32", "unit": "TFLOP/s",
            "achieved": samp_tflops, "peak": fp32_peak, "frac": samp_tflops / fp32_peak,
            "traffic": SAMPLER_TRAFFIC_BYTES,
            "algorithmic_flops_per_launch": proposals * flops_per_proposal,
            "note": (f"algorithmic flops per proposal = {SAMPLER_FLOPS_RATIO} M (ratio t0 + g t1, |.|^2, product) "
                     f"+ acceptance x {SAMPLER_FLOPS_ACCEPT} M (θ update and Möbius update of g), M = {M}, "
                     f"acceptance {m.acceptance:.3f}; {proposals} proposals per launch; peak = FP32 FMA rate of "
                     f"152 SMs x 128 lanes at the sampled SM clock ({sm_ghz:.3f} GHz), derived (MEASURED_PEAKS.json "
                     f"has no FP32 figure); the kernel keeps θ, g and σ on chip (traffic from ncu)"),
            "kernel_ms": kernels, "dominant_kernel": max(kernels, key=kernels.get),
            "share_of_three": {k: v / ksum for k, v in kernels.items()}}
    s_kernel_ms = st[7]
    s_flops = 2.0 * (2 * P) ** 2 * Ns / 2.0        # upper triangle of the 2P x 2P real Gram
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    roof["tensor_kernel"] = {
        "kernel": "gram_tf32_kernel (S = X Xᵀ, upper tiles)", "bound": "tensor",
        "achieved": s_flops / (s_kernel_ms * 1e-3) / 1e12, "peak": bf16_peak, "unit": "TFLOP/s",
        "frac": s_flops / (s_kernel_ms * 1e-3) / 1e12 / bf16_peak, "traffic": GRAM_TRAFFIC_BYTES,
        "note": "peak = measured dense bf16 burst (of measured); algorithmic flops = 2*(2P)^2*Ns/2 per launch; "
                "TF32 operands issue at half the bf16 rate"}
    issue_rate = SAMPLER_NCU["warp_instructions"] / (SAMPLER_NCU["duration_us"] * 1e-6)
    roof["sampler_issue_bound"] = {
        "bound": "instruction issue", "warp_instructions_per_launch": SAMPLER_NCU["warp_instructions"],
        "achieved": issue_rate, "peak": 152 * 4 * 2.07e9, "unit": "warp instructions/s",
        "frac": issue_rate / (152 * 4 * 2.07e9), "issue_active_pct": SAMPLER_NCU["issue_active_pct"],
        "note": (f"executed (not algorithmic) instructions over the duration of one ncu capture of this "
                 f"workload's launch (acceptance {SAMPLER_NCU['acceptance']}, "
                 f"{SAMPLER_NCU['warp_instructions_per_warp_step']} warp instructions per warp and step); "
                 f"peak = 152 SMs x 4 schedulers x 2.07 GHz")}

    line = {
        "metric": METRIC, "value": value, "unit": "SR steps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (random-init RBM weights, Philox-seeded chains)",
        "config": workload_config(),
        "precision": {"s": int(sp), "eval": int(eval_precision_choice()),
                      "note": "nq_s_precision / nq_eval_precision of the timed step (1 = TF32 S, 0 = FP32 evaluation)"},
        "clocks": clk.summary(), "e2e": e2e, "gpu_launches": int(launches),
        "effective_samples_per_s": ess, "tau_int_eloc": tau, "energy_per_site": m.mean_re / w["N"],
        "stage_ms": stages, "kernel_ms": kernels,
        "tuning": eng.tuning(),
        "s_precision_modes": modes,
        "roofline": roof,
    }
    if int(os.environ.get("RANK", "0")) == 0 and not args.no_batch:
        line["many_problems"] = batched_vs_sequential()
    if int(os.environ.get("RANK", "0")) == 0 and not args.no_precision:
        line["precision_modes"] = precision_modes()
    if int(os.environ.get("RANK", "0")) == 0 and not args.no_learned:
        line["learned_proposal"] = learned_vs_local()
    if int(os.environ.get("RANK", "0")) == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(max_seconds=args.cpu_seconds)
    return line


# --------------------------------------------------------------------------
# Learned proposal vs local Metropolis on the 6x6 transverse-field Ising model
# --------------------------------------------------------------------------
LEARNED = dict(L=6, h=3.04, J=1.0, alpha=4, chains=8192, chain_length=20, burn=50, eps=0.01, lr=0.02,
               sr_steps=100, train_every=10, train_steps=50, train_batch=4096, train_lr=1e-3, p_ar=0.5,
               ess_length=64, ess_burn=20, seed=0x4E51)


def _tfim2d(nq, Lx, h, J):
    N = Lx * Lx
    hilb = nq.HomogeneousSpin(N)
    H = nq.LocalOperator(hilb)
    for x in range(Lx):
        for y in range(Lx):
            i = x + Lx * y + 1
            H = H - h * nq.sigmax(hilb, i)
            H = H + J * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, (x + 1) % Lx + Lx * y + 1)
            H = H + J * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, x + Lx * ((y + 1) % Lx) + 1)
    return hilb, H


PRECISION = dict(N=12, alpha=2, beta=2, g=1.0, V=2.0, gamma=1.0, chains=16384, chain_length=8, burn=100,
                 eps=0.01, lr=0.01, sr_steps=20, seed=0x4E51)


def _dissipative(nq, hilb, N, g, V, gamma):
    H = nq.LocalOperator(hilb)
    Ls = []
    for i in range(1, N + 1):
        H = H + (g / 2) * nq.sigmax(hilb, i)
        Ls.append(float(np.sqrt(gamma)) * nq.sigmam(hilb, i))
    for i in range(1, N):
        H = H + (V / 4) * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i + 1)
    return nq.liouvillian(H, Ls)


def precision_modes():
    """Dissipative Ising chain N = 12 (open; g = 1, V = 2, γ = 1), NDM α = β = 2
    (P = 1248 real parameters), 16384 chains x 8 samples: on the same samples,
    the relative error of L_loc, F, S and Δw of the precision mode (FP32
    evaluation, TF32 S on tcgen05, FP32 inverse with FP64 refinement) against
    FP64 evaluation with FP32 S; then 20 SR steps of TF32 S vs FP32 S from the
    same start, comparing the cost ⟨|Lρ|²⟩/⟨ρ²⟩."""
    import nqcuda as nq
    c = PRECISION
    N = c["N"]
    hilb = nq.HomogeneousSpin(N)
    lv = _dissipative(nq, hilb, N, c["g"], c["V"], c["gamma"])

    def engine(prec, sp):
        net = nq.NDM(np.float64, N, c["alpha"], c["beta"], nq.af_softplus)
        nq.init_random_pars_(net, sigma=1e-4, rng=np.random.default_rng(c["seed"]))
        smp = nq.MetropolisSampler(nq.LocalRule(), c["chain_length"], 2 * N, burn=c["burn"], seed=c["seed"])
        return nq.BatchedSampler(net, smp, lv, nq.SR(eps=c["eps"]), batch_sz=c["chains"], eval_precision=prec,
                                 s_precision=sp).engine

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b))))

    ref = engine(nq._lib.NQ_EVAL_F64, nq._lib.NQ_S_F32)
    fast = engine(nq._lib.NQ_EVAL_F32, nq._lib.NQ_S_TF32)
    samples, _ = ref.sample(3)
    fast.set_samples(samples)
    out = {"workload": "ndm_dissipative_ising_N12_alpha2_beta2_16384x8", "n_params": ref.P}
    m0, l0, f0 = ref.estimate(want_loc=True, want_force=True)
    m1, l1, f1 = fast.estimate(want_loc=True, want_force=True)
    s0, s1 = ref.sr_matrix(), fast.sr_matrix()
    d0, d1 = ref.precondition(0, c["eps"]), fast.precondition(0, c["eps"])
    out["relative_error_vs_fp64_eval"] = {"L_loc": rel(l1, l0), "cost": abs(m1.mean_re - m0.mean_re) / abs(m0.mean_re),
                                          "F": rel(f1, f0), "S": rel(s1, s0), "dw": rel(d1, d0)}
    # the solve's own error: Δw against the FP64 solve of each engine's own S and F
    eye = np.eye(s0.shape[0])
    out["solve_error_vs_fp64_solve_of_own_S"] = {
        "fp64_eval": rel(d0, np.linalg.solve(s0 + c["eps"] * eye, f0)),
        "precision_mode": rel(d1, np.linalg.solve(s1 + c["eps"] * eye, f1))}
    out["dw_error_from_S"] = rel(np.linalg.solve(s1 + c["eps"] * eye, f1), np.linalg.solve(s0 + c["eps"] * eye, f1))
    out["solve_corrections"] = {"fp64_eval": ref.sr_info()[0],
                                "precision_mode": fast.sr_info()[0]}
    # θ of the density matrix on tcgen05: BF16 hi + lo (x2) and hi + mid + lo (x3)
    for name, prec in (("theta_bf16x2", nq._lib.NQ_EVAL_TC_BF16X2), ("theta_bf16x3", nq._lib.NQ_EVAL_TC_BF16X3)):
        e = engine(prec, nq._lib.NQ_S_TF32)
        e.set_samples(samples)
        mt, lt, ft = e.estimate(want_loc=True, want_force=True)
        st_ = e.sr_matrix()
        dt = e.precondition(0, c["eps"])
        out["relative_error_vs_fp64_eval_" + name] = {
            "L_loc": rel(lt, l0), "cost": abs(mt.mean_re - m0.mean_re) / abs(m0.mean_re), "F": rel(ft, f0),
            "S": rel(st_, s0), "dw": rel(dt, d0)}
        del e
    del ref, fast
    curves = {}
    for name, prec, sp in (("tf32", nq._lib.NQ_EVAL_F32, nq._lib.NQ_S_TF32),
                           ("fp32", nq._lib.NQ_EVAL_F32, nq._lib.NQ_S_F32),
                           ("bf16_theta_tf32_S", nq._lib.NQ_EVAL_TC_BF16X2, nq._lib.NQ_S_TF32)):
        e = engine(prec, sp)
        curves[name] = [e.vmc_step(it, c["eps"], c["lr"]).mean_re for it in range(c["sr_steps"])]
        del e
    out["cost_curve_tf32"] = curves["tf32"]
    out["cost_curve_fp32"] = curves["fp32"]
    out["cost_curve_bf16_theta_tf32_S"] = curves["bf16_theta_tf32_S"]
    out["final_cost_relative_difference"] = abs(curves["tf32"][-1] - curves["fp32"][-1]) / abs(curves["fp32"][-1])
    out["final_cost_relative_difference_bf16_theta"] = (abs(curves["bf16_theta_tf32_S"][-1] - curves["fp32"][-1]) /
                                                        abs(curves["fp32"][-1]))
    return out


BATCH = dict(n_problems=64, sizes=(3, 4, 5), h_range=(2.0, 4.0), J=1.0, alpha=1, chains=1024, chain_length=20,
             burn=50, eps=0.01, lr=0.01, seed=1, steps=10)


def _batch_problems(nq):
    """The 64 problems of the many-problem workload: (network, Hilbert space,
    Hamiltonian) per problem, drawn from the workload's seed."""
    c = BATCH
    rng = np.random.default_rng(c["seed"])
    spec = [(int(rng.choice(c["sizes"])), float(rng.uniform(*c["h_range"]))) for _ in range(c["n_problems"])]
    probs = []
    for k, (L, h) in enumerate(spec):
        hilb, H = _tfim2d(nq, L, h, c["J"])
        net = nq.RBM(np.complex64, L * L, c["alpha"], nq.af_logcosh)
        nq.init_random_pars_(net, sigma=0.01, rng=np.random.default_rng(100 + k))
        probs.append((net, hilb, H))
    return spec, probs


def batched_step(probs):
    """One batched SR step for all problems: device ms per step (10 timed
    steps after 3 + 10 warm-up steps), kernels per step and the tuning."""
    import nqcuda as nq
    c = BATCH
    batch = nq.ProblemBatch(probs, c["chains"], c["chain_length"], c["burn"])
    for i in range(3):
        batch.vmc_step(i, c["eps"], c["lr"])
    l0 = batch.kernel_launches()
    ms_b = batch.bench_steps(10, c["steps"], c["eps"], c["lr"])     # one untimed step, then the timed ones
    launches_b = (batch.kernel_launches() - l0) / (c["steps"] + 1)
    tuning = batch.tuning()
    del batch
    return float(np.mean(ms_b)), launches_b, tuning


def batched_vs_sequential():
    """64 independent 2D TFIM ground-state problems (L in {3,4,5}, h in
    U[2,4] from seed 1, J = 1, complex RBM alpha = 1, 1024 chains x 20
    samples): one batched SR step (every stage of all problems one grouped
    launch, 17 kernels) against the same 64 problems stepped one after the
    other, each replaying its own single-problem graph."""
    import nqcuda as nq
    c = BATCH
    spec, probs = _batch_problems(nq)
    ms_bat, launches_b, tuning = batched_step(probs)
    engines = []
    for k, (net, hilb, H) in enumerate(probs):
        smp = nq.MetropolisSampler(nq.LocalRule(), c["chain_length"], hilb.n_sites, burn=c["burn"],
                                   seed=0x4E51 + 7919 * k)
        engines.append(nq.BatchedSampler(net, smp, H, nq.SR(eps=c["eps"]), batch_sz=c["chains"],
                                         s_precision=nq._lib.NQ_S_TF32).engine)
    for e in engines:
        for i in range(3):
            e.vmc_step(i, c["eps"], c["lr"])
    dev_ms = sum(float(np.mean(e.bench_steps(10, 3, c["eps"], c["lr"], 0))) for e in engines)
    t0 = time.perf_counter()
    for it in range(c["steps"]):
        for e in engines:
            e.vmc_step(100 + it, c["eps"], c["lr"])
    wall_seq = (time.perf_counter() - t0) / c["steps"] * 1e3
    return {"workload": "64 x tfim2d L in {3,4,5}, h~U[2,4], rbm alpha=1, 1024 chains x 20",
            "sizes": [L for L, _ in spec], "batched_ms_per_step": ms_bat,
            "batched_problem_steps_per_s": c["n_problems"] * 1e3 / ms_bat,
            "batched_kernels_per_step": launches_b, "tuning": tuning,
            "sequential_device_ms_per_step": dev_ms,
            "sequential_wall_ms_per_step": wall_seq,
            "sequential_problem_steps_per_s": c["n_problems"] * 1e3 / wall_seq,
            "speedup_vs_sequential_wall": wall_seq / ms_bat,
            "speedup_vs_sequential_device": dev_ms / ms_bat}


def cg_step():
    """The matrix-free CG SR step (tolerance 1e-4) on the 6x6 TFIM workload
    of the learned-proposal comparison, from its random start: device ms per
    step over 5 timed steps after 3 + 10 warm-up steps, CG iterations."""
    import nqcuda as nq
    c = LEARNED
    N = c["L"] * c["L"]
    hilb, H = _tfim2d(nq, c["L"], c["h"], c["J"])
    net = nq.RBM(np.complex64, N, c["alpha"], nq.af_logcosh)
    nq.init_random_pars_(net, sigma=0.01, rng=np.random.default_rng(c["seed"]))
    smp = nq.MetropolisSampler(nq.LocalRule(), c["chain_length"], N, burn=c["burn"], seed=c["seed"])
    eng = nq.BatchedSampler(net, smp, H, nq.SR(eps=c["eps"], algorithm=nq.sr_cg, precision=1e-4),
                            batch_sz=c["chains"], s_precision=nq._lib.NQ_S_TF32).engine
    for i in range(3):
        eng.vmc_step(i, c["eps"], c["lr"])
    ms = float(np.mean(eng.bench_steps(10, 5, c["eps"], c["lr"], 0)))
    it, res = eng.sr_info()
    return {"workload": "tfim2d_6x6_h3.04_rbm_alpha4_8192_chains matrix-free CG", "ms_per_step": ms,
            "cg_iterations": it, "relative_residual": res}


def cg_ndm_step():
    """The matrix-free CG SR solve over the materialised O rows (X) against the
    direct solve on the dissipative Ising NDM workload (N = 12, α = β = 2,
    P = 1248 real parameters, 16384 chains x 8, FP32 evaluation, SR
    tolerance 1e-4): Δw of both on one sample set, then device ms per whole
    SR step over 5 timed steps after 3 + 10 warm-up steps, CG iterations."""
    import nqcuda as nq
    c = PRECISION
    N = c["N"]
    hilb = nq.HomogeneousSpin(N)
    lv = _dissipative(nq, hilb, N, c["g"], c["V"], c["gamma"])

    def engine(algorithm):
        net = nq.NDM(np.float64, N, c["alpha"], c["beta"], nq.af_softplus)
        nq.init_random_pars_(net, sigma=1e-4, rng=np.random.default_rng(c["seed"]))
        smp = nq.MetropolisSampler(nq.LocalRule(), c["chain_length"], 2 * N, burn=c["burn"], seed=c["seed"])
        return nq.BatchedSampler(net, smp, lv, nq.SR(eps=c["eps"], algorithm=algorithm, precision=1e-4),
                                 batch_sz=c["chains"]).engine

    direct, cg = engine(nq.sr_cholesky), engine(nq.sr_cg)
    samples, _ = direct.sample(3)
    cg.set_samples(samples)
    direct.estimate()
    cg.estimate()
    d0, d1 = direct.precondition(0, c["eps"]), cg.precondition(0, c["eps"])
    out = {"workload": "ndm_dissipative_ising_N12_alpha2_beta2_16384x8 SR step, direct vs matrix-free CG over X",
           "n_params": direct.P,
           "dw_relative_difference": float(np.max(np.abs(d1 - d0)) / np.max(np.abs(d0)))}
    for name, eng in (("direct", direct), ("cg", cg)):
        for i in range(3):
            eng.vmc_step(i, c["eps"], c["lr"])
        out[name + "_ms_per_step"] = float(np.mean(eng.bench_steps(10, 5, c["eps"], c["lr"], 0)))
    it, res = cg.sr_info()
    out["cg_iterations"], out["relative_residual"] = it, res
    return out


def learned_vs_local():
    """SR on the 6x6 TFIM (h = 3.04) with the MADE proposal trained online on
    the chains' samples every 10 SR steps, then effective samples/s of local
    Metropolis and of the 50/50 mixture at several sweep lengths (passes).
    ESS = samples / tau_int with tau_int = 1 + 2 Σ ρ (Sokal window) of E_loc
    and of |Σσz| per chain; the sampling time is the sampler stage's device
    time.  Energies of both samplers are reported with their difference."""
    import nqcuda as nq
    from nqcuda.stats import integrated_autocorr_time, autocorrelation
    c = LEARNED
    N = c["L"] * c["L"]
    hilb, H = _tfim2d(nq, c["L"], c["h"], c["J"])
    net = nq.RBM(np.complex64, N, c["alpha"], nq.af_logcosh)
    nq.init_random_pars_(net, sigma=0.01, rng=np.random.default_rng(c["seed"]))
    smp = nq.MetropolisSampler(nq.LocalRule(), c["chain_length"], N, burn=c["burn"], seed=c["seed"])
    eng = nq.BatchedSampler(net, smp, H, nq.SR(eps=c["eps"]), batch_sz=c["chains"],
                            s_precision=nq._lib.NQ_S_TF32).engine
    eng.proposal_init(128, 0.0, c["seed"])
    t0 = time.perf_counter()
    nll = []
    for it in range(c["sr_steps"]):
        m = eng.vmc_step(it, c["eps"], c["lr"])
        if it % c["train_every"] == c["train_every"] - 1:
            nll.append(eng.proposal_train(c["train_steps"], c["train_batch"], c["train_lr"]))
    wall = time.perf_counter() - t0
    params = eng.get_params()
    made = eng.proposal_get_params()
    sr_ms = float(np.mean(eng.bench_steps(1000, 5, c["eps"], 0.0, L2_FLUSH_BYTES)))
    del eng
    # the same SR step with the matrix-free conjugate-gradient solve (no S)
    smp_cg = nq.MetropolisSampler(nq.LocalRule(), c["chain_length"], N, burn=c["burn"], seed=c["seed"])
    cg = nq.BatchedSampler(net, smp_cg, H, nq.SR(eps=c["eps"], algorithm=nq.sr_cg, precision=1e-4),
                           batch_sz=c["chains"]).engine
    cg.set_params(params)
    cg_ms = float(np.mean(cg.bench_steps(1000, 5, c["eps"], 0.0, L2_FLUSH_BYTES)))
    cg_iters, cg_res = cg.sr_info()
    del cg

    def measure(p_ar, passes):
        s2 = nq.MetropolisSampler(nq.LocalRule(), c["ess_length"], passes, burn=c["ess_burn"], seed=c["seed"] + 1)
        e = nq.BatchedSampler(net, s2, H, nq.SR(eps=c["eps"]), batch_sz=c["chains"],
                              s_precision=nq._lib.NQ_S_TF32).engine
        e.set_params(params)
        if p_ar > 0:
            e.proposal_init(128, 0.0, c["seed"])
            e.proposal_set_params(made)
            e.proposal_set_mix(p_ar)
        e.sample(5000, want_samples=False)          # warm-up (autotuner, first launch)
        smp_, _ = e.sample(5001)
        ms = float(e.stage_times()[0])
        mm, loc, _ = e.estimate(want_loc=True)
        mz = np.abs(smp_.sum(axis=2)).astype(np.float64)
        tE = integrated_autocorr_time(loc.T)
        tM = integrated_autocorr_time(mz.T)
        rhoE = autocorrelation(loc.T, 40)
        r = {"passes": e.passes, "sample_ms": ms, "tau_E": tE, "tau_absM": tM,
             "ess_per_s_E": loc.size / tE / (ms * 1e-3), "ess_per_s_absM": loc.size / tM / (ms * 1e-3),
             "energy_per_site": mm.mean_re / N, "energy_err_per_site": mm.error / N}
        if p_ar > 0:
            a, b = e.proposal_stats()
            r["ar_acceptance"] = b / max(a, 1)
        r["_rhoE"] = rhoE
        del e
        return r

    local = [measure(0.0, p) for p in (1, 3, 9, N)]
    mixed = [measure(c["p_ar"], p) for p in (1, 3)]
    bl = max(local, key=lambda r: r["ess_per_s_E"])
    bm = max(mixed, key=lambda r: r["ess_per_s_E"])
    # Ceiling of the 50/50 mixture on this configuration, whatever the cost
    # of an AR move: at one step per sample (the mixture's best spacing) half
    # of the steps are local moves, so a step costs at least half a local
    # step; an AR step can at most replace the state by an independent draw,
    # so ρ_mix(k) >= (1/2)^k ρ_L(k) (every one of the k steps local) and
    # τ_mix >= 1 + 2 Σ_k (1/2)^k ρ_L(k) ("perfect proposal").  With the trained
    # proposal's measured τ_mix in place of that bound, the same formula
    # gives the ceiling of this proposal at zero AR cost.
    l1 = local[0]
    ns_e = c["chains"] * c["ess_length"]
    rho = l1["_rhoE"]
    tau_perfect = 1.0 + 2.0 * float(sum(0.5 ** k * rho[k] for k in range(1, len(rho))))
    half_step_s = 0.5 * l1["sample_ms"] * 1e-3
    steps_per_chain = c["ess_length"] + c["ess_burn"]
    ceiling = {
        "tau_E_local_one_step": l1["tau_E"], "tau_E_mixture_measured": mixed[0]["tau_E"],
        "tau_E_mixture_perfect_proposal_bound": tau_perfect,
        "ess_ratio_ceiling_zero_ar_cost_measured_proposal": ns_e / mixed[0]["tau_E"] / half_step_s / bl["ess_per_s_E"],
        "ess_ratio_ceiling_zero_ar_cost_perfect_proposal": ns_e / tau_perfect / half_step_s / bl["ess_per_s_E"],
        "local_step_ns": l1["sample_ms"] * 1e6 / (c["chains"] * steps_per_chain),
        "mixture_step_ns": mixed[0]["sample_ms"] * 1e6 / (c["chains"] * steps_per_chain),
    }
    ceiling["ar_move_ns"] = 2 * ceiling["mixture_step_ns"] - ceiling["local_step_ns"]
    for r in local + mixed:
        r.pop("_rhoE", None)
    return {"workload": "tfim2d_6x6_h3.04_rbm_alpha4_8192_chains", "sr_ms_per_step": sr_ms,
            "sr_steps_per_s": 1e3 / sr_ms,
            "matrix_free_cg": {"sr_ms_per_step": cg_ms, "sr_steps_per_s": 1e3 / cg_ms, "iterations": cg_iters,
                               "relative_residual": cg_res, "tolerance": 1e-4},
            "training_wall_s": wall, "energy_per_site_after_sr": m.mean_re / N,
            "made_nll_after_each_training": nll, "local": local, "learned_mixture": mixed,
            "best_local_ess_per_s_E": bl["ess_per_s_E"], "best_learned_ess_per_s_E": bm["ess_per_s_E"],
            "learned_over_local_ess_ratio": bm["ess_per_s_E"] / bl["ess_per_s_E"],
            "mixture_ceiling": ceiling,
            "abs_dE_per_site_learned_vs_local": abs(bm["energy_per_site"] - bl["energy_per_site"])}


# --------------------------------------------------------------------------
# CPU reference arm: the oracle port (FP64 restatement of the reference path)
# --------------------------------------------------------------------------
def cpu_baseline(max_seconds=20.0, chains=None):
    """Times the oracle's restatement of one reference VMC iteration on a
    bounded number of chains and scales to the full workload, on all host
    cores and, in a separate process limited to one thread (OpenMP and
    BLAS), on one core."""
    from oracle import cport
    res = cport.time_baseline(WORKLOAD, max_seconds=max_seconds, chains=chains, precision="f32")
    f64 = cport.time_baseline(WORKLOAD, max_seconds=max_seconds / 2, chains=chains, precision="f64")
    res["fp64"] = {"value": f64["value"], "unit": f64["unit"], "cores": f64["cores"], "sample": f64["sample"]}
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1", MKL_NUM_THREADS="1")
    code = ("import json; from oracle import cport; "
            f"w = json.loads({json.dumps(json.dumps(WORKLOAD))}); "
            f"print(json.dumps(cport.time_baseline(w, max_seconds={max_seconds / 2!r}, quiet=True, "
            f"precision='f32')))")
    try:
        out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                             timeout=max(120.0, 6 * max_seconds), cwd=os.path.dirname(os.path.abspath(__file__)))
        one = json.loads(out.stdout.strip().splitlines()[-1])
        res["single_core"] = {"value": one["value"], "unit": one["unit"], "cores": 1, "sample": one["sample"]}
    except (subprocess.SubprocessError, ValueError, IndexError, KeyError) as e:
        res["single_core"] = {"unavailable": f"{type(e).__name__}"}
    return res


def run_reference(args):
    from oracle import cport
    # each step is a bounded sample of the workload, sized so that the whole
    # run stays within about three minutes
    per_step = min(args.cpu_seconds, max(2.0, 180.0 / (args.steps + args.warmup)))
    res = []
    for _ in range(args.warmup):
        cport.time_baseline(WORKLOAD, max_seconds=per_step / 4, quiet=True, precision="f32")
    for _ in range(args.steps):
        res.append(cport.time_baseline(WORKLOAD, max_seconds=per_step, precision="f32"))
    v = float(np.median([r["value"] for r in res]))
    base = res[-1]
    base["value"] = v
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "SR steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / v, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
            "config": workload_config(), "cpu_baseline": base,
            "e2e": {"value": v, "unit": "SR steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def aggregate_replicas(line, world):
    """N independent replicas (one per GPU, "scaling": "weak"): the whole-job
    throughput is N steps per slowest rank's step time, for the device-timed
    value and for e2e.  Collective over the default process group."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([line["ms_per_step"], -line["e2e"]["value"]], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    line["ms_per_step"] = float(t[0])
    line["value"] = world * 1e3 / line["ms_per_step"]
    line["e2e"]["value"] = world * float(-t[1])
    line["n_gpus"] = world
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the 64-problem batched vs sequential comparison")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the precision-mode comparison (NDM N=12)")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-proposal vs local Metropolis comparison (6x6 TFIM)")
    ap.add_argument("--batch-only", action="store_true",
                    help="time only the batched step of the 64-problem workload (for launch lists)")
    ap.add_argument("--cg-only", action="store_true",
                    help="time only the matrix-free CG SR step of the 6x6 TFIM workload (for profiles)")
    ap.add_argument("--cg-ndm-only", action="store_true",
                    help="time only the direct and the matrix-free CG SR steps of the N=12 NDM workload")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.cg_only:
        print(json.dumps(cg_step()))
        return
    if args.cg_ndm_only:
        print(json.dumps(cg_ndm_step()))
        return
    if args.batch_only:
        import nqcuda as nq
        _, probs = _batch_problems(nq)
        ms, kernels, tuning = batched_step(probs)
        print(json.dumps({"workload": "64 x tfim2d batched step", "batched_ms_per_step": ms,
                          "batched_kernels_per_step": kernels, "tuning": tuning}))
        return
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args)))
        return
    barrier = None
    if world > 1:
        # one replica per GPU: the library sees only this rank's device
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ.get("LOCAL_RANK", str(rank))
        import torch.distributed as dist
        dist.init_process_group("gloo")
        barrier = dist.barrier
        if rank != 0:
            args.no_cpu_baseline = args.no_learned = args.no_batch = args.no_precision = True
    line = run_gb300(args, barrier)
    if world > 1:
        import torch.distributed as dist
        aggregate_replicas(line, world)
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
