"""nqcuda -- host side of libnqcuda, the GB300 (sm_103a) engine for the
variational Monte Carlo step of NeuralQuantum.jl.

The names mirror the reference API (Julia's ``f!`` becomes ``f_``; lattice
sites are 1-based as in the reference).  Every numerical stage runs in
libnqcuda; importing this package does not load it, the first engine does.
"""
from ._lib import build, lib, NqError  # noqa: F401
from . import _lib  # noqa: F401
from .hilbert import HomogeneousSpin, HomogeneousFock, SuperOpSpace, physical, nsites  # noqa: F401
from .operators import (LocalOperator, KLocalOperator, KLocalOperatorSum, KLocalLiouvillian,  # noqa: F401
                        sigmax, sigmay, sigmaz, sigmam, sigmap, liouvillian, op_table)
from .networks import RBM, NDM, NDMSymm, RBMSplit, af_logcosh, af_softplus, init_random_pars_  # noqa: F401
from .networks import Dense, WSum, Chain, PureStateAnsatz, PureChain, sum_autobatch, identity  # noqa: F401
from .networks import DenseSplit, PositiveDefR, MixedStateAnsatz  # noqa: F401
from .samplers import MetropolisSampler, ExactSampler, LocalRule, ExchangeRule, OperatorRule  # noqa: F401
from .stats import Measurement  # noqa: F401
from .iterative import (BatchedSampler, BatchedObsKetSampler, BatchedObsDMSampler, add_observable_,  # noqa: F401
                        compute_observables, SR, Descent, sample_,  # noqa: F401
                        precondition_, update_,  # noqa: F401
                        sr_shift, sr_multiplicative, sr_none, sr_cholesky, sr_cg, sr_minres, sr_qlp, sr_lsq,
                        sr_diag, sr_div)
from .engine import Engine, ProblemBatch  # noqa: F401
from .lattice import HyperCube, translational_symm_table, quantum_ising_hamiltonian, lattice_average_operator  # noqa: F401,E501
