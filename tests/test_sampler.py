"""The host-side restatement of HMMER's profile sampling chain
(p7_hmm_Sample -> p7_ProfileConfig -> mf_conversion, p7_Lambda) against the
reference-generated golden profiles: identical rbv bytes, byte costs, scale
and lambda. (mu needs MSV scores; its GPU check is in test_gpu_batch.py.)"""
import glob
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
# sampled-profile cases (mM_sSEED); the tut_* cases are models read from HMM files
CASES = sorted(os.path.basename(p)[:-5] for p in glob.glob(os.path.join(GOLDEN, "m*_s*.prof")))


@pytest.mark.parametrize("name", CASES)
def test_sampled_profile_equals_reference(name):
    ref = F.read_profile(os.path.join(GOLDEN, name + ".prof"))
    seed = int(name.split("_s")[1])
    got = api.sample_profile(ref.M, seed)
    assert np.array_equal(got.rbv, ref.rbv)
    assert (got.tbm_b, got.tec_b, got.base_b, got.bias_b) == (ref.tbm_b, ref.tec_b, ref.base_b, ref.bias_b)
    assert np.float32(got.scale_b) == np.float32(ref.scale_b)
    assert np.float32(got.mlambda) == np.float32(ref.mlambda)


def test_sampler_rejects_bad_arguments():
    with pytest.raises(api.MSVError):
        api.sample_profile(0, 1)
