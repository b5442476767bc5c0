"""The vectorized CPU port (the timed baseline) against the reference's
golden vectors and against the scalar oracle: bit-exact status, score and
pass flag."""
import glob
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import formats as F
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.res")))


@pytest.mark.parametrize("name", CASES)
def test_port_matches_reference(name):
    p = F.read_profile(os.path.join(GOLDEN, name + ".prof"))
    s = F.read_seqs(os.path.join(GOLDEN, name + ".seqs"))
    r = F.read_results(os.path.join(GOLDEN, name + ".res"))
    o, used = O.port_batch(p, s, nthreads=2)
    assert used == 2
    assert np.array_equal(o["status"], r.status)
    assert np.array_equal(o["sc"].view(np.uint32), r.sc.view(np.uint32))
    assert np.array_equal(o["pass"], r.passed)


def test_port_matches_oracle_on_random_profiles():
    rng = np.random.default_rng(5)
    for M in (1, 16, 17, 100, 333):
        costs = rng.integers(0, 60, size=(F.KP_AMINO, M)).astype(np.uint8)
        p = F.profile_from_node_costs(costs, tbm_b=int(rng.integers(5, 60)), tec_b=3, base_b=190,
                                      bias_b=int(rng.integers(5, 50)), scale_b=4.328085, mmu=-9.0, mlambda=0.69)
        s = F.synth_sequences(150, seed=M, lmax=2000)
        a = O.msv_batch(p, s, nthreads=2)
        b, _ = O.port_batch(p, s, nthreads=2)
        assert np.array_equal(a["status"], b["status"])
        assert np.array_equal(a["sc"].view(np.uint32), b["sc"].view(np.uint32))
        assert np.array_equal(a["pass"], b["pass"])
