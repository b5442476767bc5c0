"""The ViterbiFilter oracle (oracle/vit_oracle.c) against p7_ViterbiFilter's
own golden results: every status and every score bit pattern, for sampled
models in hmmsearch's local mode and the tutorial Pfam models."""
import glob
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import formats as F
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
VIT = sorted(os.path.basename(p)[4:-6] for p in glob.glob(os.path.join(GOLDEN, "vit_*.vprof")))


def test_golden_set_is_complete():
    assert len(VIT) >= 14


@pytest.mark.parametrize("name", VIT)
def test_oracle_reproduces_reference_viterbi_filter(name):
    vp = F.read_vprofile(os.path.join(GOLDEN, "vit_" + name + ".vprof"))
    s = F.read_seqs(os.path.join(GOLDEN, name + ".seqs"))
    st, sc = F.read_vresults(os.path.join(GOLDEN, "vit_" + name + ".vres"))
    o = O.vit_batch(vp, s)
    assert np.array_equal(o["status"], st)
    ok = st >= 0
    assert np.array_equal(o["sc"][ok].view(np.uint32), sc[ok].view(np.uint32))


def test_golden_covers_overflow_and_the_dd_paths():
    n_erange = 0
    for name in VIT:
        st, _ = F.read_vresults(os.path.join(GOLDEN, "vit_" + name + ".vres"))
        n_erange += int((st == 16).sum())
    assert n_erange >= 5


def test_crop_vprofile_keeps_the_nodes():
    """A profile cut at its own length is the profile (the striping helper
    the per-width GPU parity cases use)."""
    from tests.vprofiles import crop_vprofile
    for name in ("m777_s3", "m2400_s1", "m17_s2"):
        vp = F.read_vprofile(os.path.join(GOLDEN, "vit_" + name + ".vprof"))
        same = crop_vprofile(vp, vp.M)
        assert np.array_equal(same.rwv, vp.rwv) and np.array_equal(same.twv, vp.twv)
