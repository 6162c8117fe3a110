"""FP64 CPU oracle for the NeuralQuantum.jl variational Monte Carlo step.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (the ``nqcuda`` host package
or ``libnqcuda``) imports this package; only ``tests/``, the smoke entry point
and the CPU-baseline and reference legs of ``bench.py`` use it, to check and
to time the GPU path, never as part of it.

Each module restates one part of the reference algorithm in plain numpy
(float64 / complex128) and cites the reference file:line it follows:

* ``philox``      -- Philox4x32-10 counter-based RNG (Salmon et al., SC'11) and
                     the counter schema shared with the CUDA sampler.
* ``hilbert``     -- spin / Fock encodings, ``local_index``, ``set!``
                     (src/Hilbert/HomogeneousSpin.jl, HomogeneousFock.jl,
                     SuperHilbert.jl, DoubledHilbert.jl).
* ``operators``   -- k-local operators as row tables, sums, products,
                     adjoints, the Liouvillian super-operator
                     (src/Operators/...).
* ``networks``    -- RBM and NDM log-amplitudes and gradients in the
                     reference flat parameter order (src/Networks/...).
* ``sampler``     -- Metropolis local-flip replay (src/Samplers/Metropolis.jl).
* ``estimators``  -- local energy / Liouvillian estimators and the cost
                     gradient (src/IterativeInterface/...).
* ``sr``          -- SR S/F set-up, shifted Cholesky solve, Descent update
                     (src/Algorithms/SR/SRDirect.jl, src/Optimisers/).
* ``stats``       -- ``Measurement`` statistics (src/utils/stats.jl).
* ``exact``       -- exact enumeration helpers for small systems.

Parity pinning: the reference is Julia and cannot be executed here (no Julia
runtime), and it stores no golden numeric vectors.  The oracle is pinned
instead to the reference's own known answers and test properties: the exact
ground-state energies quoted in examples/ising1d.jl:46-47 and
examples/ising2d.jl:55 (the 5 x 5 lattice, by the Lanczos recurrence of
lanczos.c),
the operator/Liouvillian matrix conventions of test/Operators/ising.jl:28-42
(rebuilt here from independent Kronecker products), hand-written gradients
against numerical differentiation (test/Machines/test_grad.jl:108-138), and
the sampler chi-square test of test/Samplers/test_samplers.jl:26-31.
"""
