"""Host-side logic (CPU only): the C-ABI library exports, operator
flattening against the oracle, golden fixtures, and API validation that
needs no GPU."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

import nqcuda as nq
from nqcuda import _lib
from oracle import operators as oops, exact as oex, networks as onw, estimators as oest
from oracle.hilbert import Hilbert, SPIN, FOCK

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")


def declared_symbols():
    src = open(os.path.join(REPO, "include", "nqcuda.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nq_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_loads_and_exports_every_declared_symbol():
    nq.build()
    L = ctypes.CDLL(_lib.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 18
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) <= set(_lib.EXPORTS), set(syms) - set(_lib.EXPORTS)
    lib = nq.lib()
    assert lib.nq_abi_version() == 1
    assert b"sm_103a" in lib.nq_version()


def test_create_rejects_bad_config_without_touching_the_gpu():
    lib = nq.lib()
    cfg = _lib.NqConfig()
    cfg.network = 7
    h = ctypes.c_void_p()
    assert lib.nq_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.NQ_ERR_ARG
    assert not h.value
    assert lib.nq_create(None, ctypes.byref(h)) == _lib.NQ_ERR_ARG
    # the diagonal sampler space is defined for the NDM only; unknown spaces are refused
    for net, space in ((_lib.NQ_NET_RBM, _lib.NQ_SPACE_DIAGONAL), (_lib.NQ_NET_NDM, 5)):
        cfg = _lib.NqConfig()
        cfg.network, cfg.activation, cfg.hilbert = net, _lib.NQ_ACT_SOFTPLUS, _lib.NQ_HILB_FOCK
        cfg.n_sites, cfg.n_hidden, cfg.n_ancilla, cfg.n_chains, cfg.chain_length, cfg.passes = 4, 4, 4, 16, 2, 1
        cfg.sampler_space = space
        assert lib.nq_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.NQ_ERR_ARG
        assert not h.value


def test_config_layout_matches_header():
    """nq_config keeps the C layout of include/nqcuda.h: sampler_space takes
    the first reserved word, the size is unchanged."""
    assert ctypes.sizeof(_lib.NqConfig) == 88
    assert _lib.NqConfig.sampler_space.offset == 76


def _random_configs(n, N, kind, rng):
    vals = [-1, 1] if kind == "spin" else [0, 1]
    return rng.choice(vals, size=(n, N))


@pytest.mark.parametrize("kind", ["spin", "fock"])
def test_ket_op_table_matches_oracle_connections(kind):
    N, h_, J = 7, 0.8, 1.3
    hilb = nq.HomogeneousSpin(N) if kind == "spin" else nq.HomogeneousFock(N)
    H = nq.LocalOperator(hilb)
    for i in range(1, N + 1):
        H -= h_ * nq.sigmax(hilb, i)
        H += J * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i % N + 1)
    tab = nq.op_table(H)
    ohilb = Hilbert(N, SPIN if kind == "spin" else FOCK)
    oH = oex.tfim_1d(ohilb, h_, J)
    rng = np.random.default_rng(0)
    for cfg in _random_configs(50, N, kind, rng):
        a = tab.connections(cfg)
        b = oops.connections_ket(oH, cfg.astype(float))
        assert len(a) == len(b)
        for (ma, ca), (mb, cb) in zip(a, b):
            assert abs(ma - mb) < 1e-14
            assert sorted(ca) == sorted((s, int(v)) for s, v in cb)


def test_liouvillian_op_table_matches_oracle_connections():
    N, g, V = 5, 1.0, 2.0
    hilb = nq.HomogeneousFock(N)
    H = nq.LocalOperator(hilb)
    Ls = []
    for i in range(1, N + 1):
        H += g / 2 * nq.sigmax(hilb, i)
        Ls.append(nq.sigmam(hilb, i))
    for i in range(1, N):
        H += V / 4 * nq.sigmaz(hilb, i) * nq.sigmaz(hilb, i + 1)
    lv = nq.liouvillian(H, Ls)
    tab = nq.op_table(lv)
    ohilb = Hilbert(N, FOCK)
    oH, oL = oex.dissipative_ising(ohilb, g, V)
    olv = oops.liouvillian(oH, oL)
    rng = np.random.default_rng(1)
    for _ in range(40):
        s = rng.integers(0, 2, N)
        e = rng.integers(0, 2, N)
        a = tab.connections(np.concatenate([s, e]))
        b = oops.connections_doubled(olv, s.astype(float), e.astype(float))
        assert len(a) == len(b)
        for (ma, ca), (mb, cl, cr) in zip(a, b):
            assert abs(ma - mb) < 1e-14
            ref = [(s_, int(v)) for s_, v in cl] + [(s_ + N, int(v)) for s_, v in cr]
            assert sorted(ca) == sorted(ref)


def test_golden_rbm_fixture_pins_the_oracle():
    fx = json.load(open(os.path.join(GOLDEN, "rbm_logpsi.json")))
    r = onw.RBM(fx["N"], fx["M"], onw.LOGCOSH)
    r.set_flat(np.array(fx["params_re"]) + 1j * np.array(fx["params_im"]))
    st = np.array(fx["states"], dtype=float)
    lp = r.logpsi(st)
    assert np.allclose(lp.real, fx["logpsi_re"], atol=1e-12)
    assert np.allclose(lp.imag, fx["logpsi_im"], atol=1e-12)
    H = oex.tfim_1d(Hilbert(fx["N"], SPIN), 1.0, 1.0)
    E = oest.local_energy(r, H, st)
    assert np.allclose(E.real, fx["eloc_re"], atol=1e-12)


def test_host_api_mirrors_reference_names():
    for name in ("BatchedSampler", "MetropolisSampler", "LocalRule", "RBM", "NDM", "SR",
                 "Descent", "sample_", "precondition_", "update_", "sigmax", "sigmaz", "sigmam",
                 "liouvillian", "LocalOperator", "init_random_pars_", "HomogeneousSpin",
                 "HomogeneousFock", "BatchedObsKetSampler", "BatchedObsDMSampler", "ExactSampler",
                 "ExchangeRule", "add_observable_", "compute_observables"):
        assert hasattr(nq, name), name
    s = nq.MetropolisSampler(nq.LocalRule(), 20, 20, burn=50)
    assert s.passes == 21        # Metropolis.jl:30-38
    with pytest.raises(ValueError):
        nq.sigmax(nq.HomogeneousSpin(4), 5)


def test_hypercube_and_lattice_operators():
    """HyperCube.jl:26-136 and SimpleOperators.jl:160-185: edges (u < v, in
    the reference's SimpleGraph order), translations as circshift of the
    column-major vertex grid, and the quantum Ising Hamiltonian of an open
    chain equal to the oracle's g/2 Σσx + V/4 Σσzσz."""
    from oracle import exact as oex, operators as oops
    assert nq.HyperCube([4]).edges() == [(1, 2), (1, 4), (2, 3), (3, 4)]
    assert nq.HyperCube([4], periodic=False).edges() == [(1, 2), (2, 3), (3, 4)]
    sq = nq.HyperCube([3, 3])
    assert sq.nv() == 9 and sq.ne() == 18 and sq.vert_coords[1] == [2, 1]
    assert nq.HyperCube([2, 3], periodic=[False, True]).ne() == 3 + 6
    assert nq.translational_symm_table(nq.HyperCube([4])) == [[1, 2, 3, 4], [4, 1, 2, 3], [3, 4, 1, 2],
                                                               [2, 3, 4, 1]]
    t2 = nq.translational_symm_table(sq)
    assert len(t2) == 9 and t2[1] == [7, 8, 9, 1, 2, 3, 4, 5, 6] and t2[3] == [3, 1, 2, 6, 4, 5, 9, 7, 8]
    N = 4
    hilb = nq.HomogeneousFock(N)
    H = nq.quantum_ising_hamiltonian(nq.HyperCube([N], periodic=False), hilb, g=1.0, V=2.0)
    oh = Hilbert(N, FOCK)
    oH, _ = oex.dissipative_ising(oh, 1.0, 2.0)
    tab = nq.op_table(H)
    dense = np.zeros((oh.dim, oh.dim), complex)
    for i, st in enumerate(oh.all_states()):
        for mel, ch in tab.connections(st):
            s2 = st.copy()
            for site, v in ch:
                s2[site] = v
            dense[i, oh.index_of_state(s2[None])[0]] += mel
    np.testing.assert_allclose(dense, oops.to_matrix(oH), atol=1e-12)
    avg = nq.lattice_average_operator(nq.HyperCube([N]), hilb, nq.sigmaz)
    assert len(nq.op_table(avg).connections(oh.all_states()[0])) >= 1
    perms = nq.translational_symm_table(nq.HyperCube([N]))
    net = nq.NDMSymm(np.float64, N, 1, 1, perms)
    assert net.permutations.min() == 0 and net.permutations.max() == N - 1


def test_product_path_never_reaches_the_oracle():
    """The host package and the CUDA sources neither import nor load anything
    from oracle/: the oracle is the checker of the tests, the smoke entry point
    and the bench's CPU legs, never part of the path it checks."""
    import re
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    pkg = os.path.join(root, "neuralquantum.jl_gb300")
    pat = re.compile(r"(import\s+oracle|from\s+oracle|oracle[/\\]|libnqport|cport)")
    hits = []
    for d, _, files in os.walk(pkg):
        if "_build" in d or "__pycache__" in d:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".c", ".cpp")):
                path = os.path.join(d, f)
                with open(path, encoding="utf-8") as fh:
                    for n, line in enumerate(fh, 1):
                        if pat.search(line):
                            hits.append(f"{os.path.relpath(path, root)}:{n}: {line.strip()}")
    assert not hits, hits


def test_positive_def_r_host_layer_and_chain_validation():
    """PositiveDefR (Layers/PositiveDefR.jl): real Wr, Wi, b; the chain's flat
    vector carries them with zero imaginary part, later complex layers keep
    theirs; the layer is nq_layer kind 4 and opens density-matrix chains only
    (checked by the Python mirror and by nq_create_chain before any device
    call)."""
    N, M = 4, 6
    l0 = nq.PositiveDefR(np.float32, N, M, nq.af_logcosh, rng=np.random.default_rng(1))
    assert l0.Wr.dtype == np.float32 and l0.Wi.shape == (M, N) and l0.b.shape == (M,)
    with pytest.raises(ValueError):
        nq.PositiveDefR(np.complex64, N, M)
    net = nq.MixedStateAnsatz(nq.Chain(l0, nq.Dense(np.complex64, M, 3, nq.af_softplus), nq.WSum(np.complex64, 3)),
                              N)
    assert net.real_sr
    nq.init_random_pars_(net, sigma=0.1, rng=np.random.default_rng(2))
    p = net.flat()
    n1 = 2 * M * N + M
    assert p.dtype == np.complex128 and np.all(p[:n1].imag == 0) and np.any(p[n1:].imag != 0)
    assert np.all(p[:n1].real != 0)
    net.set_flat(p + 1j)
    np.testing.assert_array_equal(net.flat()[:n1], p[:n1])
    arr = nq.engine.chain_layers(net)
    assert [a.kind for a in arr] == [_lib.NQ_LAYER_POSITIVE_DEF_R, _lib.NQ_LAYER_DENSE, _lib.NQ_LAYER_WSUM]
    with pytest.raises(ValueError):
        nq.MixedStateAnsatz(nq.Chain(nq.Dense(np.complex64, N, M), l0, nq.sum_autobatch), N)
    lib = nq.lib()
    cases = [
        (_lib.NQ_NET_MIXED_CHAIN, [(_lib.NQ_LAYER_DENSE_SPLIT, N, M, 0), (_lib.NQ_LAYER_POSITIVE_DEF_R, M, M, 0),
                                   (_lib.NQ_LAYER_SUM, M, 1, 0)]),
        (_lib.NQ_NET_CHAIN, [(_lib.NQ_LAYER_POSITIVE_DEF_R, N, M, 0), (_lib.NQ_LAYER_SUM, M, 1, 0)]),
    ]
    for network, layers in cases:
        cfg = _lib.NqConfig()
        cfg.network, cfg.hilbert = network, _lib.NQ_HILB_SPIN
        cfg.n_sites, cfg.n_chains, cfg.chain_length, cfg.passes = N, 16, 2, 1
        arr = (_lib.NqLayer * len(layers))(*[_lib.NqLayer(*l) for l in layers])
        h = ctypes.c_void_p()
        assert lib.nq_create_chain(ctypes.byref(cfg), len(layers), arr, ctypes.byref(h)) == _lib.NQ_ERR_ARG
        assert not h.value
