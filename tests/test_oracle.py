"""Pins the FP64 oracle to the reference's known answers and test properties
(CPU only)."""
import json
import os

import numpy as np
import pytest

from oracle import philox, operators as ops, networks as nw, exact, sampler as osm, stats as ost, \
    estimators as oest, sr as osr
from oracle.hilbert import Hilbert, SPIN, FOCK

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_philox_known_answers():
    """Random123 known-answer vectors of Philox4x32-10."""
    kat = json.load(open(os.path.join(GOLDEN, "philox_kat.json")))
    for case in kat:
        r = philox.philox4x32_10(*case["ctr"], *case["key"])
        assert [int(x) for x in r] == case["out"]


@pytest.mark.parametrize("kind", [SPIN, FOCK])
def test_operator_and_liouvillian_matrices(kind):
    """test/Operators/ising.jl:5-42: H and the Liouvillian from the row
    tables equal independently built dense operators (N=4, g=0.7, V=2)."""
    N, g, V = 4, 0.7, 2.0
    h = Hilbert(N, kind)
    H = ops.OpSum(h)
    Ls = []
    for i in range(N):
        H = H + ops.sigmax(h, i).scale(g / 2)
        Ls.append(ops.sigmam(h, i))
    for i in range(N):
        H = H + ops.prod(ops.sigmaz(h, i), ops.sigmaz(h, (i + 1) % N)).scale(V / 4)
    sx = np.array([[0, 1], [1, 0]]); sz = np.diag([1.0, -1.0]); sm = np.array([[0, 0], [1, 0.0]])
    Hq = sum(g / 2 * ops.embed(h, i, sx) for i in range(N)) + \
        sum(V / 4 * ops.embed(h, i, sz) @ ops.embed(h, (i + 1) % N, sz) for i in range(N))
    assert np.abs(ops.to_matrix(H) - Hq).max() < 1e-12
    Lq = [ops.embed(h, i, sm) for i in range(N)]
    assert np.abs(ops.liouvillian_to_matrix(ops.liouvillian(H, [])) - ops.dense_liouvillian(Hq, [])).max() < 1e-12
    assert np.abs(ops.liouvillian_to_matrix(ops.liouvillian(ops.OpSum(h), Ls)) -
                  ops.dense_liouvillian(0 * Hq, Lq)).max() < 1e-12
    assert np.abs(ops.liouvillian_to_matrix(ops.liouvillian(H, Ls)) - ops.dense_liouvillian(Hq, Lq)).max() < 1e-12


def test_row_table_conventions():
    """Diagonal always stored (KLocalOperator.jl:76-80), σz = diag(+1,-1) on
    local index (0,1) (SimpleOperators.jl:55-65), σ⁻ maps index 0 -> 1."""
    h = Hilbert(2, SPIN)
    sx = ops.sigmax(h, 0)
    assert sx.conns[0][0][0] == 0 and sx.conns[0][0][1] == []
    assert sx.conns[0][1][1] == [(0, 1.0)]
    sz = ops.sigmaz(h, 1)
    assert sz.conns[0][0][0] == 1 and sz.conns[1][0][0] == -1
    sm = ops.sigmam(h, 0)
    assert sm.conns[0] == [[0j, []]] and sm.conns[1][1][1] == [(0, -1.0)]


def test_known_ground_energy_1d():
    """examples/ising1d.jl:46-47: E0 = -1.274549484318 * 20 for
    H = -Σσx + Σσzσz, N=20, periodic."""
    kat = json.load(open(os.path.join(GOLDEN, "known_answers.json")))
    e = exact.tfim_ground_energy_1d(20, 1.0, 1.0)
    assert abs(e / 20 - kat["tfim1d_N20_h1_J1_energy_per_site"]) < 1e-9


def test_known_ground_energy_2d():
    """examples/ising2d.jl:55 quotes E0 = -80.13310152422413 for the 5 x 5
    periodic TFIM at h = 3.  The matrix-free Lanczos on the oracle's tfim_2d
    convention reproduces it to 1e-9 with the coupling sign J = -1
    (ferromagnetic, H = -h Σσx - Σσzσz); the example's code adds +J σzσz,
    whose frustrated (odd L) ground energy is -79.6241413371 instead.  The
    convention itself is pinned by dense diagonalisation of the oracle's
    operator tables at 3 x 3 for both signs."""
    kat = json.load(open(os.path.join(GOLDEN, "known_answers.json")))
    h9 = Hilbert(9, SPIN)
    for J in (1.0, -1.0):
        e_dense = np.linalg.eigvalsh(ops.to_matrix(exact.tfim_2d(h9, 3, 3, 3.0, J)).real)[0]
        assert abs(exact.tfim_ground_energy_2d(3, 3, 3.0, J) - e_dense) < 1e-9
        assert abs(exact.tfim_ground_energy_2d(3, 3, 3.0, J, z2=False) - e_dense) < 1e-9
    e = exact.tfim_ground_energy_2d(5, 5, 3.0, -1.0, iters=80)
    assert abs(e - kat["tfim2d_5x5_h3_J1_energy"]) < 1e-9


def test_oracle_hamiltonian_matches_lanczos_convention():
    N = 8
    h = Hilbert(N, SPIN)
    H = exact.tfim_1d(h, 1.0, 1.0)
    e_dense = np.linalg.eigvalsh(ops.to_matrix(H).real)[0]
    assert abs(e_dense - exact.tfim_ground_energy_1d(N, 1.0, 1.0)) < 1e-9


@pytest.mark.parametrize("act", [nw.LOGCOSH, nw.SOFTPLUS])
def test_gradients_vs_finite_differences(act):
    """test/Machines/test_grad.jl:108-138 (hand-written gradient == AD)."""
    rng = np.random.default_rng(0)
    N = 4
    r = nw.RBM(N, 2 * N, act)
    nw.init_random_pars(r, rng, sigma=0.2 ** 2)
    n = nw.NDM(N, 1, 2, act)
    nw.init_random_pars(n, rng, sigma=0.2 ** 2)
    sp = nw.RBMSplit(N, 2 * N, act)
    nw.init_random_pars(sp, rng, sigma=0.2 ** 2)
    s = rng.choice([-1.0, 1.0], size=(3, N))
    sr = rng.choice([0.0, 1.0], size=(3, N)); sc = rng.choice([0.0, 1.0], size=(3, N))
    for net, f, args in ((r, r.logpsi, (s,)), (n, n.logpsi, (sr, sc)), (sp, sp.logpsi, (sr, sc))):
        _, g = net.logpsi_and_grad(*args)
        p = net.flat()
        eps = 1e-6
        for k in range(p.size):
            q = p.copy(); q[k] += eps; net.set_flat(q); lp = f(*args)
            q[k] -= 2 * eps; net.set_flat(q); lm = f(*args)
            assert np.max(np.abs((lp - lm) / (2 * eps) - g[:, k])) < 1e-7
        net.set_flat(p)


def test_rbmsplit_is_the_rbm_of_the_doubled_sites():
    """RBMSplit.jl:48-50: logρ(σ, η) equals an RBM over the 2N sites (σ, η)
    with a = (ar, ac) and W = (Wr | Wc); the flat vectors coincide
    (ar, ac, b, Wr, Wc column-major = a, b, W column-major)."""
    rng = np.random.default_rng(12)
    N, M = 3, 5
    sp = nw.RBMSplit(N, M, nw.LOGCOSH)
    nw.init_random_pars(sp, rng, sigma=0.3 ** 2)
    r = nw.RBM(2 * N, M, nw.LOGCOSH)
    r.set_flat(sp.flat())
    np.testing.assert_array_equal(r.a, np.concatenate([sp.ar, sp.ac]))
    np.testing.assert_array_equal(r.W, np.concatenate([sp.Wr, sp.Wc], axis=1))
    sr = rng.choice([-1.0, 1.0], size=(7, N)); sc = rng.choice([-1.0, 1.0], size=(7, N))
    v = np.concatenate([sr, sc], axis=1)
    np.testing.assert_allclose(sp.logpsi(sr, sc), r.logpsi(v), rtol=0, atol=1e-13)
    np.testing.assert_allclose(sp.logpsi_and_grad(sr, sc)[1], r.logpsi_and_grad(v)[1], rtol=0, atol=1e-13)


def test_ndm_symm_restatement():
    """NDMSymm (NDMSymm.jl): with the identity as the only permutation the
    bare NDM is the symmetric one (up to the averaged visible biases); the
    bare logρ is invariant under relabelling the sites by a permutation of
    the group when the group is closed (translations of a ring), and the
    symmetrised gradient equals finite differences of logρ in the symmetric
    parameters along directions that keep the visible biases uniform."""
    rng = np.random.default_rng(14)
    N = 4
    trans = [[(i + t) % N for i in range(N)] for t in range(N)]
    ns = nw.NDMSymm(N, 2, 1, trans, nw.LOGCOSH)
    v = rng.standard_normal(ns.n_params) * 0.3
    ns.set_flat(v)
    assert ns.bare.Mh == 2 * N and ns.bare.Ma == N
    sr = rng.choice([0.0, 1.0], size=(5, N)); sc = rng.choice([0.0, 1.0], size=(5, N))
    shift = [(i + 1) % N for i in range(N)]
    np.testing.assert_allclose(ns.logpsi(sr, sc), ns.logpsi(sr[:, shift], sc[:, shift]), atol=1e-12)
    one = nw.NDMSymm(N, 2, 1, [list(range(N))], nw.LOGCOSH)
    one.set_flat(v)
    np.testing.assert_allclose(one.bare.flat(), one.sym.flat(), atol=0)
    _, g = ns.logpsi_and_grad(sr, sc)
    p0 = ns.flat()
    eps = 1e-6
    for k in range(p0.size):
        d = np.zeros_like(p0)
        d[k] = 1.0
        o = 0
        for f in nw.NDM.FIELDS:
            n = int(np.prod(ns.sym.shapes[f]))
            if f in ("b_mu", "b_la") and o <= k < o + n:
                d[o:o + n] = 1.0 / N          # a uniform visible-bias direction
            o += n
        ns.set_flat(p0 + eps * d); lp = ns.logpsi(sr, sc)
        ns.set_flat(p0 - eps * d); lm = ns.logpsi(sr, sc)
        fd = (lp - lm) / (2 * eps)
        assert np.max(np.abs(fd - g @ d)) < 1e-7, k
    ns.set_flat(p0)


@pytest.mark.parametrize("layers", [
    [("dense", 4, 8, nw.LOGCOSH), ("sum", 8)],
    [("dense", 4, 8, nw.IDENTITY), ("dense", 8, 12, nw.IDENTITY), ("wsum", 12)],
    [("dense", 4, 3, nw.SOFTPLUS), ("dense", 3, 2, nw.SOFTPLUS), ("wsum", 2)],
    [("dense", 4, 8, nw.LOGCOSH), ("dense", 8, 4, nw.LOGCOSH), ("sum", 4)]])
def test_chain_gradients_vs_finite_differences(layers):
    """The chains of test/Machines/test_grad.jl:29-44 and test_batched.jl:
    32-46: backprop gradient == finite differences (holomorphic), and a
    single Dense + sum is the RBM without visible bias."""
    rng = np.random.default_rng(3)
    N = 4
    ch = nw.Chain(N, layers)
    nw.init_random_pars(ch, rng, sigma=0.3 ** 2)
    s = rng.choice([-1.0, 1.0], size=(5, N))
    _, g = ch.logpsi_and_grad(s)
    p = ch.flat()
    eps = 1e-6
    for k in range(p.size):
        q = p.copy(); q[k] += eps; ch.set_flat(q); lp = ch.logpsi(s)
        q[k] -= 2 * eps; ch.set_flat(q); lm = ch.logpsi(s)
        assert np.max(np.abs((lp - lm) / (2 * eps) - g[:, k])) < 1e-7
    ch.set_flat(p)
    if layers[0][3] == nw.LOGCOSH and len(layers) == 2:
        r = nw.RBM(N, 8, nw.LOGCOSH)
        r.W, r.b = ch.params[0][0], ch.params[0][1]
        np.testing.assert_allclose(ch.logpsi(s), r.logpsi(s), atol=1e-13)


def test_ndm_parameter_count():
    n = nw.NDM(6, 1, 1)
    assert n.n_params == 2 * 6 + 2 * 6 + 6 + 2 * 36 + 2 * 36


def test_stats_matches_formula():
    rng = np.random.default_rng(1)
    v = rng.standard_normal((16, 10)) + 1j * rng.standard_normal((16, 10))
    st = ost.stat_analysis(v)
    assert abs(st["mean"] - v.mean()) < 1e-12
    mc = v.mean(1)
    assert abs(st["error"] - np.sqrt(np.var(mc, ddof=1) / 16)) < 1e-12


def test_sampler_replay_is_deterministic_and_detailed_balance():
    """χ² of the replayed local-flip chain against exact |ψ|² (N=4)."""
    from scipy.stats import chisquare
    rng = np.random.default_rng(5)
    h = Hilbert(4, SPIN)
    r = nw.RBM(4, 4, nw.LOGCOSH)
    nw.init_random_pars(r, rng, sigma=0.2 ** 2)
    s1, _ = osm.run(r.log_prob, h, 4096, 1, 20, 5, seed=9)
    s2, _ = osm.run(r.log_prob, h, 4096, 1, 20, 5, seed=9)
    np.testing.assert_array_equal(s1, s2)
    idx = h.index_of_state(s1.reshape(-1, 4))
    counts = np.bincount(idx, minlength=16)
    p = exact.ket_distribution(r, h)
    assert chisquare(counts, p * counts.sum())[1] >= 0.01


def hopping_field(h, N, t=1.0, g=0.4):
    """Σ_i t(σ⁺_i σ⁻_{i+1} + σ⁻_i σ⁺_{i+1}) + g Σ_i σx_i on an open chain:
    rows of the hopping terms have 1 or 2 connections, so the OperatorRule's
    factor n(σ)/n(σ') is not 1; the field makes the moves ergodic."""
    H = ops.OpSum(h)
    for i in range(N - 1):
        H = H + ops.prod(ops.sigmap(h, i), ops.sigmam(h, i + 1)).scale(t)
        H = H + ops.prod(ops.sigmam(h, i), ops.sigmap(h, i + 1)).scale(t)
    for i in range(N):
        H = H + ops.sigmax(h, i).scale(g)
    return H


def test_operator_rule_replay_detailed_balance():
    """χ² of the OperatorRule replay (OperatorRule.jl:42-58, with the factor
    n(σ)/n(σ')) against exact |ψ|², on an operator with rows of unequal
    length; without the factor the chain is biased."""
    from scipy.stats import chisquare
    rng = np.random.default_rng(8)
    N = 4
    h = Hilbert(N, SPIN)
    r = nw.RBM(N, 4, nw.LOGCOSH)
    nw.init_random_pars(r, rng, sigma=0.3 ** 2)
    H = hopping_field(h, N)
    lens = {len(ops.connections_ket(H, s)) for s in h.all_states()}
    assert len(lens) > 1
    s1, info = osm.run(r.log_prob, h, 3000, 1, 40, 5, seed=3, move_op=H)
    idx = h.index_of_state(s1.reshape(-1, N))
    counts = np.bincount(idx, minlength=h.dim)
    p = exact.ket_distribution(r, h)
    assert chisquare(counts, p * counts.sum())[1] >= 0.01
    assert 0 < info["accepted"] < info["steps"]


def test_local_energy_sums_to_exact_expectation():
    """<E_loc>_{|ψ|²} over all states equals <ψ|H|ψ>/<ψ|ψ>."""
    rng = np.random.default_rng(2)
    h = Hilbert(5, SPIN)
    r = nw.RBM(5, 5, nw.LOGCOSH)
    nw.init_random_pars(r, rng, sigma=0.3 ** 2)
    H = exact.tfim_1d(h, 1.0, 1.0)
    st = h.all_states()
    E = oest.local_energy(r, H, st)
    p = exact.ket_distribution(r, h)
    assert abs(np.sum(p * E) - exact.exact_local_energy_expectation(r, H)) < 1e-10


def test_liouvillian_local_values_exact():
    """L_loc(σ,η) = (L ρ)(σ,η)/ρ(σ,η) against the dense super-operator
    (idea of test/Problems/problem_algs.jl:23-30)."""
    rng = np.random.default_rng(4)
    N = 3
    h = Hilbert(N, FOCK)
    n = nw.NDM(N, 1, 1, nw.SOFTPLUS)
    nw.init_random_pars(n, rng, sigma=0.3 ** 2)
    H, Ls = exact.dissipative_ising(h, 1.0, 2.0)
    lv = ops.liouvillian(H, Ls)
    st = h.all_states()
    D = h.dim
    sr = np.repeat(st[None], D, axis=0).reshape(-1, N)
    sc = np.repeat(st, D, axis=0)
    rho = np.exp(n.logpsi(sr, sc))
    Lm = ops.liouvillian_to_matrix(lv)
    Lrho = Lm @ rho
    L, _ = oest.local_liouvillian(n, lv, sr, sc, with_grad=False)
    assert np.max(np.abs(L - Lrho / rho)) < 1e-9


@pytest.mark.parametrize("kind", [SPIN, FOCK])
def test_dm_local_observables_sum_to_trace(kind):
    """Σ_σ ρ(σ,σ) O_loc(σ) / Tr ρ equals the dense Tr(ρ Ô)/Tr(ρ) for the
    diagonal-chain estimator of BatchedObsDMSampler.jl:90-105, and ρ is
    Hermitian with a real, positive diagonal."""
    rng = np.random.default_rng(6)
    N = 3
    h = Hilbert(N, kind)
    n = nw.NDM(N, 1, 2, nw.SOFTPLUS)
    nw.init_random_pars(n, rng, sigma=0.4 ** 2)
    rho = exact.density_matrix(n, h)
    assert np.max(np.abs(rho - rho.conj().T)) < 1e-12
    assert np.all(np.diag(rho).real > 0) and np.max(np.abs(np.diag(rho).imag)) < 1e-12
    p = exact.diagonal_distribution(n, h)
    np.testing.assert_allclose(p, np.diag(rho).real / np.trace(rho).real, rtol=1e-12)
    st = h.all_states()
    cases = [ops.OpSum(h) + ops.sigmax(h, 0) + ops.sigmax(h, 2),
             ops.OpSum(h) + ops.prod(ops.sigmay(h, 0), ops.sigmay(h, 1)),
             ops.OpSum(h) + ops.prod(ops.sigmaz(h, 1), ops.sigmam(h, 2)),
             ops.OpSum(h) + ops.sigmaz(h, 1)]
    for O in cases:
        loc = oest.local_observable_dm(n, O, st)
        assert abs(np.sum(p * loc) - exact.dm_expectation(n, O)) < 1e-10


def test_sr_algorithms_and_the_multiplicative_quirk():
    """SRDirect.jl:51-90: for a positive-definite shifted S, sr_diag (pinv),
    sr_cholesky and sr_div agree; the reference's sr_cholesky / sr_div solve
    with S itself under sr_multiplicative (the shift reaches sr_diag only)."""
    rng = np.random.default_rng(9)
    O = rng.standard_normal((300, 10)) + 1j * rng.standard_normal((300, 10))
    S = osr.build_S(O - O.mean(0), real_params=False)
    F = rng.standard_normal(10) + 1j * rng.standard_normal(10)
    ref = osr.precondition(S, F, 0.01)
    for alg in ("diag", "div"):
        np.testing.assert_allclose(osr.precondition(S, F, 0.01, algorithm=alg), ref, rtol=1e-10, atol=1e-12)
    q = osr.precondition(S, F, 0.01, kind="multiplicative", it=3, follow_reference=True)
    np.testing.assert_allclose(q, osr.precondition(S, F, 0.01, kind="none"), rtol=1e-10, atol=1e-12)
    d = osr.precondition(S, F, 0.01, kind="multiplicative", it=3, algorithm="diag", follow_reference=True)
    np.testing.assert_allclose(d, osr.precondition(S, F, 0.01, kind="multiplicative", it=3), rtol=1e-10,
                               atol=1e-12)


def test_sr_solve_matches_direct():
    rng = np.random.default_rng(3)
    O = rng.standard_normal((200, 12)) + 1j * rng.standard_normal((200, 12))
    E = rng.standard_normal(200) + 0j
    Oc, _ = oest.center(O)
    S = osr.build_S(Oc, False)
    F = oest.force_ket(E, O)
    dw = osr.precondition(S, F, 0.01)
    assert np.allclose((S + 0.01 * np.eye(12)) @ dw, F)


def test_c_port_matches_numpy_oracle():
    """The C restatement (timed CPU baseline) reproduces the numpy oracle:
    identical Philox chains and the same E_loc / Δw."""
    from oracle import cport
    N, M, B, L, burn, passes, seed = 6, 12, 32, 3, 4, 7, 99
    h = Hilbert(N, SPIN)
    H = exact.tfim_1d(h, 1.0, 1.0)
    r = nw.RBM(N, M, nw.LOGCOSH)
    nw.init_random_pars(r, np.random.default_rng(8), sigma=0.2 ** 2)
    port = cport.PortRBM(N, M, nw.LOGCOSH, SPIN, H)
    newp, samples, E, dw = port.iteration(r.flat(), B, L, burn, passes, seed, 3, 0.01, 0.1)
    ref, info = osm.run(r.log_prob, h, B, L, burn, passes, seed, call=3)
    np.testing.assert_array_equal(samples, ref)
    flat = ref.reshape(-1, N)
    Eo = oest.local_energy(r, H, flat)
    assert np.max(np.abs(E - Eo)) < 1e-10
    _, O = r.logpsi_and_grad(flat)
    Oc, _ = oest.center(O)
    dwo = osr.precondition(osr.build_S(Oc, False), oest.force_ket(Eo, O), 0.01)
    assert np.max(np.abs(dw - dwo)) < 1e-8 * max(1, np.max(np.abs(dwo)))


def test_made_oracle_gradient_mask_and_normalisation():
    """MADE oracle: q sums to 1 over the space, the NLL gradient matches
    central differences, and masked weights get a zero gradient."""
    from oracle import made as om
    N = 5
    m = om.MADE(N, 128, rng=np.random.default_rng(1))
    rng = np.random.default_rng(2)
    m.b1, m.b2, m.b3 = rng.standard_normal(128) * 0.3, rng.standard_normal(128) * 0.3, rng.standard_normal(N)
    allx = om.bits_to_x(np.arange(2 ** N, dtype=np.uint64), N)
    assert abs(np.exp(m.logq(allx)).sum() - 1.0) < 1e-12
    x = allx[rng.integers(0, 2 ** N, size=40)]
    _, g = m.nll_grad(x)
    p0 = m.flat()
    for k in rng.choice(p0.size, 25, replace=False):
        e = np.zeros_like(p0)
        e[k] = 1e-6
        m.set_flat(p0 + e)
        fp = m.nll_grad(x)[0]
        m.set_flat(p0 - e)
        fm = m.nll_grad(x)[0]
        m.set_flat(p0)
        assert abs((fp - fm) / 2e-6 - g[k]) < 1e-6
    M1, M2, M3 = om.masks(N, 128)
    mask = np.concatenate([M1.ravel(), np.ones(128), M2.ravel(), np.ones(128), M3.ravel(), np.ones(N)])
    assert np.all(g[mask == 0] == 0)


def test_made_bf16_rounding_matches_torch():
    """The inference copy rounds like a float32 -> bfloat16 conversion."""
    torch = pytest.importorskip("torch")
    from oracle import made as om
    v = np.random.default_rng(0).standard_normal(10000).astype(np.float32) * 3
    v[:4] = [1.00390625, 1.01171875, -1.00390625, 0.0]        # exact ties either way
    ref = torch.tensor(v).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(om.to_bf16(v), ref)


def test_mixture_oracle_with_exact_proposal_always_accepts():
    """With q equal to the normalised |ψ|² every AR move is accepted, so the
    mixture replay's AR bookkeeping and acceptance ratio are consistent."""
    from oracle import made as om
    N, B = 4, 16
    h = Hilbert(N, SPIN)
    r = nw.RBM(N, 8, nw.LOGCOSH)
    nw.init_random_pars(r, np.random.default_rng(5), sigma=0.3 ** 2)

    class ExactQ:
        def __init__(self):
            allx = om.bits_to_x(np.arange(2 ** N, dtype=np.uint64), N)
            lp = r.log_prob(2 * allx - 1)
            self.lq = lp - np.log(np.sum(np.exp(lp)))

        def logq(self, x):
            return self.lq[om.x_to_bits(x).astype(np.int64)]

        def sample_with_uniforms(self, u):
            cdf = np.cumsum(np.exp(self.lq))
            idx = np.minimum(np.searchsorted(cdf, u[:, 0]), 2 ** N - 1)
            return om.bits_to_x(idx.astype(np.uint64), N)

    _, info = om.run_mixture(r.log_prob, h, ExactQ(), 1.0, B, 3, 2, 3, 17, call=1)
    assert info["ar"] == info["steps"]
    assert info["ar_accepted"] == info["ar"]


def test_exact_sampler_oracle_chi_square():
    """Inverse-CDF draws of the exact-sampler replay follow |ψ|² (N=4)."""
    from scipy.stats import chisquare
    from oracle import exact as oex, networks as onw, sampler as osm
    from oracle.hilbert import Hilbert, SPIN
    hilb = Hilbert(4, SPIN)
    net = onw.RBM(4, 8, onw.LOGCOSH)
    onw.init_random_pars(net, np.random.default_rng(2), sigma=0.3 ** 2)
    p = oex.ket_distribution(net, hilb)
    idx, ties = osm.exact_run(p, 256, 40, seed=9, call=3)
    counts = np.bincount(idx.ravel(), minlength=hilb.dim)
    stat, pval = chisquare(counts, p * counts.sum())
    assert pval > 1e-3 and ties == 0
    # stale-last-slot bookkeeping: slot L-1 keeps the previous contents
    prev = np.full((5, 8), -7)
    idx2, _ = osm.exact_run(p, 8, 5, seed=9, call=3, stale_last_slot=True, prev_samples=prev)
    assert np.all(idx2[4] == -7) and np.array_equal(idx2[:4], osm.exact_run(p, 8, 5, seed=9, call=3)[0][:4])


def test_batched_estimators_match_per_sample_forms():
    """The sample-batched estimators (used on the full-size sample sets) visit
    the same connections as the per-sample restatements: E_loc, F and S of a
    TFIM ket, L_loc, the cost, F and <O> of a dissipative Liouvillian."""
    rng = np.random.default_rng(12)
    N = 6
    h = Hilbert(N, SPIN)
    r = nw.RBM(N, 12, nw.LOGCOSH)
    nw.init_random_pars(r, rng, sigma=0.2 ** 2)
    H = exact.tfim_1d(h, 0.7, 1.0)
    samples = h.value(rng.integers(0, 2, size=(300, N)))
    E = oest.local_energy(r, H, samples)
    Eb = oest.local_energy_batched(r, H, samples, chunk=97)
    np.testing.assert_allclose(Eb, E, rtol=0, atol=1e-12)
    _, O = r.logpsi_and_grad(samples)
    gf = lambda a, b: r.logpsi_and_grad(samples[a:b])[1]
    np.testing.assert_allclose(oest.force_ket_batched(E, gf, 300, chunk=64), oest.force_ket(E, O),
                               rtol=0, atol=1e-12)
    Sb, _ = oest.sr_matrix_batched(gf, 300, False, chunk=64)
    np.testing.assert_allclose(Sb, osr.build_S(oest.center(O)[0], False), rtol=0, atol=1e-12)

    hf = Hilbert(4, FOCK)
    n = nw.NDM(4, 1, 1, nw.SOFTPLUS)
    nw.init_random_pars(n, rng, sigma=0.3 ** 2)
    Hd, Ls = exact.dissipative_ising(hf, 1.0, 2.0)
    lv = ops.liouvillian(Hd, Ls)
    sr = hf.value(rng.integers(0, 2, size=(200, 4)))
    sc = hf.value(rng.integers(0, 2, size=(200, 4)))
    L, dL = oest.local_liouvillian(n, lv, sr, sc)
    _, On = n.logpsi_and_grad(sr, sc)
    C, F = oest.force_liouvillian(L, dL, On)
    Lb, Cb, Fb, mOb = oest.liouvillian_force_batched(n, lv, sr, sc, chunk=77)
    np.testing.assert_allclose(Lb, L, rtol=0, atol=1e-12)
    assert abs(Cb - C) < 1e-12 * max(1.0, C)
    np.testing.assert_allclose(Fb, F, rtol=0, atol=1e-11)
    np.testing.assert_allclose(mOb, On.mean(axis=0), rtol=0, atol=1e-12)


def test_stats_centred_merge_matches_formula_at_large_offset():
    """The block-centred merge of chain means (Chan et al.) that the device
    statistics follow gives stats.jl's variance of the chain means also when
    the spread (1e-6) is tiny next to the mean (-40), where Σ|μ_c|² - B|μ|²
    cancels."""
    rng = np.random.default_rng(3)
    B, L = 1000, 9
    v = -40.0 + 1e-6 * (rng.standard_normal((B, L)) + 1j * rng.standard_normal((B, L)))
    mu_c = v.mean(axis=1)
    blocks = [mu_c[i:i + 64] for i in range(0, B, 64)]
    n, m, m2 = 0.0, 0.0 + 0j, 0.0
    for blk in blocks:
        nb, mb = len(blk), blk.mean()
        m2b = np.sum(np.abs(blk - mb) ** 2)
        if n == 0:
            n, m, m2 = nb, mb, m2b
            continue
        tot = n + nb
        d = mb - m
        m = m + d * nb / tot
        m2 = m2 + m2b + abs(d) ** 2 * n * nb / tot
        n = tot
    direct = np.sum(np.abs(mu_c - mu_c.mean()) ** 2)
    assert abs(m2 - direct) < 1e-9 * direct
    naive = np.sum(np.abs(mu_c) ** 2) - B * abs(mu_c.mean()) ** 2
    assert abs(naive - direct) > 1e-3 * direct          # the cancelling form is visibly off
    st = ost.stat_analysis(v)
    assert abs(st["error"] - np.sqrt(direct / (B - 1) / B)) < 1e-9 * st["error"]


def test_c_port_fp32_matches_oracle_within_fp32():
    """The FP32 build of the C restatement (the reference's default complex64
    precision) gives the oracle's chains and E_loc within FP32 rounding."""
    from oracle import cport
    N, M, B, L, burn, passes, seed = 6, 12, 32, 3, 4, 7, 99
    h = Hilbert(N, SPIN)
    H = exact.tfim_1d(h, 1.0, 1.0)
    r = nw.RBM(N, M, nw.LOGCOSH)
    nw.init_random_pars(r, np.random.default_rng(8), sigma=0.2 ** 2)
    port = cport.PortRBM(N, M, nw.LOGCOSH, SPIN, H, precision="f32")
    newp, samples, E, dw = port.iteration(r.flat(), B, L, burn, passes, seed, 3, 0.01, 0.1)
    ref, info = osm.run(r.log_prob, h, B, L, burn, passes, seed, call=3)
    np.testing.assert_array_equal(samples, ref)
    Eo = oest.local_energy(r, H, ref.reshape(-1, N))
    assert np.max(np.abs(E - Eo)) < 2e-5 * np.max(np.abs(Eo))


def test_mixed_chain_is_the_dense_split_formula():
    """The density-matrix chain MixedStateAnsatz(Chain(DenseSplit(N, M, f),
    sum_autobatch), N) of test/Machines/test_grad.jl:49-50: logρ(σ, η) =
    Σ_h f(Wr_h·σ + Wc_h·η + b_h) (DenseSplit.jl:11 with sum.jl), and the
    analytic gradient against central finite differences."""
    rng = np.random.default_rng(21)
    N, M = 4, 8
    mc = nw.MixedChain(N, [("dense_split", N, M, nw.SOFTPLUS), ("sum", M)])
    p = (rng.standard_normal(mc.n_params) + 1j * rng.standard_normal(mc.n_params)) * 0.3
    mc.set_flat(p)
    Wr, Wc, b = mc.dense_split()
    h = Hilbert(N, SPIN)
    sr = h.value(rng.integers(0, 2, size=(20, N)))
    sc = h.value(rng.integers(0, 2, size=(20, N)))
    direct = nw.softplus(sr @ Wr.T + sc @ Wc.T + b[None, :]).sum(axis=1)
    np.testing.assert_allclose(mc.logpsi(sr, sc), direct, rtol=0, atol=1e-12)
    lp, g = mc.logpsi_and_grad(sr, sc)
    eps = 1e-6
    for k in range(0, mc.n_params, 5):
        q = p.copy(); q[k] += eps
        mc.set_flat(q); up = mc.logpsi(sr, sc)
        q[k] -= 2 * eps
        mc.set_flat(q); dn = mc.logpsi(sr, sc)
        np.testing.assert_allclose(g[:, k], (up - dn) / (2 * eps), rtol=0, atol=1e-7)
    mc.set_flat(p)


def test_mixed_chain_positive_def_r_formula_and_gradient():
    """PositiveDefR opening a density-matrix chain (Layers/PositiveDefR.jl:11-12):
    logρ(σ, η) = Σ_h f(Wr_h·(σ + η) + i Wi_h·(σ − η) + b_h) with real Wr, Wi,
    b, then a complex Dense layer and WSum; the gradient with respect to each
    parameter (real for PositiveDefR, holomorphic for the later complex
    layers) against central finite differences."""
    rng = np.random.default_rng(23)
    N, M = 4, 6
    mc = nw.MixedChain(N, [("positive_def_r", N, M, nw.LOGCOSH), ("sum", M)])
    nw_ = M * N
    p = np.zeros(mc.n_params, np.complex128)
    p[:] = rng.standard_normal(mc.n_params) * 0.3
    mc.set_flat(p)
    Wr = p[:nw_].real.reshape(M, N, order="F")
    Wi = p[nw_:2 * nw_].real.reshape(M, N, order="F")
    b = p[2 * nw_:].real
    h = Hilbert(N, SPIN)
    sr = h.value(rng.integers(0, 2, size=(20, N)))
    sc = h.value(rng.integers(0, 2, size=(20, N)))
    direct = nw.logcosh((sr + sc) @ Wr.T + 1j * ((sr - sc) @ Wi.T) + b[None, :]).sum(axis=1)
    np.testing.assert_allclose(mc.logpsi(sr, sc), direct, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(mc.flat(), p)
    lp, g = mc.logpsi_and_grad(sr, sc)
    eps = 1e-6
    for k in range(mc.n_params):
        q = p.copy(); q[k] += eps
        mc.set_flat(q); up = mc.logpsi(sr, sc)
        q[k] -= 2 * eps
        mc.set_flat(q); dn = mc.logpsi(sr, sc)
        np.testing.assert_allclose(g[:, k], (up - dn) / (2 * eps), rtol=1e-6, atol=1e-7)
    mc.set_flat(p)
    # later complex layers: holomorphic derivative
    mc2 = nw.MixedChain(N, [("positive_def_r", N, M, nw.SOFTPLUS), ("dense", M, 3, nw.LOGCOSH), ("wsum", 3)])
    p2 = rng.standard_normal(mc2.n_params) * 0.3 + 0j
    n1 = 2 * nw_ + M
    p2[n1:] += 1j * rng.standard_normal(mc2.n_params - n1) * 0.3
    mc2.set_flat(p2)
    _, g2 = mc2.logpsi_and_grad(sr, sc)
    for k in range(0, mc2.n_params, 3):
        q = p2.copy(); q[k] += eps
        mc2.set_flat(q); up = mc2.logpsi(sr, sc)
        q[k] -= 2 * eps
        mc2.set_flat(q); dn = mc2.logpsi(sr, sc)
        np.testing.assert_allclose(g2[:, k], (up - dn) / (2 * eps), rtol=1e-6, atol=1e-7)
