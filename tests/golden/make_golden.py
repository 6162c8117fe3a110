"""Writes the golden fixtures of tests/golden/.

* philox_kat.json   -- known-answer vectors of Philox4x32-10 published with
                       the Random123 library (Salmon et al., SC'11); checked
                       against oracle/philox.py.
* known_answers.json -- exact values quoted by the reference: the 1D TFIM
                       ground-state energy per site (examples/ising1d.jl:46-47)
                       and the 2D 5x5 value (examples/ising2d.jl:55).
* rbm_logpsi.json   -- logψ and E_loc of a fixed small RBM computed by the
                       FP64 oracle, pinning the oracle against regressions.

Run from the repository root: python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import networks as nw, exact, estimators as oest  # noqa: E402
from oracle.hilbert import Hilbert, SPIN  # noqa: E402

PHILOX_KAT = [
    {"ctr": [0, 0, 0, 0], "key": [0, 0],
     "out": [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]},
    {"ctr": [0xffffffff] * 4, "key": [0xffffffff, 0xffffffff],
     "out": [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]},
    {"ctr": [0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], "key": [0xa4093822, 0x299f31d0],
     "out": [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]},
]

KNOWN = {
    "tfim1d_N20_h1_J1_energy_per_site": -1.274549484318,
    "tfim2d_5x5_h3_J1_energy": -80.13310152422413,
}


def rbm_fixture():
    rng = np.random.default_rng(20261203)
    N = 6
    h = Hilbert(N, SPIN)
    r = nw.RBM(N, 12, nw.LOGCOSH)
    nw.init_random_pars(r, rng, sigma=0.2 ** 2)
    st = h.all_states()[::5]
    H = exact.tfim_1d(h, 1.0, 1.0)
    lp = r.logpsi(st)
    E = oest.local_energy(r, H, st)
    p = r.flat()
    return {"N": N, "M": 12, "activation": "logcosh", "params_re": p.real.tolist(),
            "params_im": p.imag.tolist(), "states": st.astype(int).tolist(),
            "logpsi_re": lp.real.tolist(), "logpsi_im": lp.imag.tolist(),
            "eloc_re": E.real.tolist(), "eloc_im": E.imag.tolist()}


if __name__ == "__main__":
    json.dump(PHILOX_KAT, open(os.path.join(HERE, "philox_kat.json"), "w"), indent=1)
    json.dump(KNOWN, open(os.path.join(HERE, "known_answers.json"), "w"), indent=1)
    json.dump(rbm_fixture(), open(os.path.join(HERE, "rbm_logpsi.json"), "w"))
    print("golden fixtures written")
