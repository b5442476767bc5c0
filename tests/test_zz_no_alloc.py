"""The allocation-free search entry point, msvgb_search_static, called through
the C ABI. It exists for callers that cannot allocate device memory while they
run (their GPU memory belongs to another allocator, or allocation is banned
after start-up); it keeps its scratch in a static device array instead.

Checked against the ordinary entry point, msvgb_search, on the same inputs:
MSV results are integers, so the outputs must be identical (bit-exact), on two
calls in a row (the shared array keeps the first call's contents), and after a
call on a different database. This file is collected last on purpose."""
import ctypes
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _search_static(prof, db, out, stream):
    d_xj = out.data_ptr()
    d_fl = out.data_ptr() + db.n
    return api.lib().msvgb_search_static(prof.h, db.h, 0.02, ctypes.c_void_p(d_xj), ctypes.c_void_p(d_fl),
                                         ctypes.c_void_p(stream))


def test_search_static_equals_search_on_two_calls():
    import torch
    ctx = api.Context(0)
    p = F.read_profile(os.path.join(GOLDEN, "m400_s1.prof"))
    s1 = F.SeqSet.concat([F.synth_sequences(3000, seed=91, lmax=6000), F.emit_homologs(p, 60, seed=92),
                          F.SeqSet.from_list([np.zeros(0, np.uint8)])])
    s2 = F.SeqSet.concat([F.synth_sequences(1500, seed=93, lmax=2000), F.emit_homologs(p, 30, seed=94, repeat=20)])
    prof = api.DeviceProfile(ctx, p)
    db1, db2 = api.DeviceDB(ctx, s1), api.DeviceDB(ctx, s2)
    want1 = api.search(ctx, prof, db1)
    want2 = api.search(ctx, prof, db2)

    stream = torch.cuda.Stream()
    out1 = torch.zeros(2 * db1.n, dtype=torch.uint8, device="cuda")   # caller-owned outputs
    out2 = torch.zeros(2 * db2.n, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        out1.fill_(0x5A)
        torch.cuda.synchronize()
        assert _search_static(prof, db1, out1, stream.cuda_stream) == api.eslOK
        stream.synchronize()
        got = out1.cpu().numpy()
        assert np.array_equal(got[:db1.n], want1[0])
        assert np.array_equal(got[db1.n:], want1[1])
    assert _search_static(prof, db2, out2, stream.cuda_stream) == api.eslOK
    assert _search_static(prof, db1, out1, stream.cuda_stream) == api.eslOK
    stream.synchronize()
    assert np.array_equal(out2.cpu().numpy(), np.concatenate(want2))
    assert np.array_equal(out1.cpu().numpy(), np.concatenate(want1))
    ctx.close()


def test_search_static_rejects_sequences_over_its_limit():
    import torch
    ctx = api.Context(0)
    p = F.read_profile(os.path.join(GOLDEN, "m200_s1.prof"))
    limit = 65535
    s = F.SeqSet.from_list([np.ones(limit + 1, np.uint8), np.ones(10, np.uint8)])
    prof, db = api.DeviceProfile(ctx, p), api.DeviceDB(ctx, s)
    out = torch.zeros(2 * db.n, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    assert _search_static(prof, db, out, 0) == api.eslEINVAL
    assert b"MSVGB_STATIC_MAX_LEN" in api.lib().msvgb_last_error()
    ctx.close()


def test_search_static_allocates_nothing_after_its_first_call():
    """The defining property: once the first call on a device has looked up
    the static array (and the runtime has loaded the kernel), further calls
    leave the device's free memory exactly where it was."""
    import torch
    ctx = api.Context(0)
    p = F.read_profile(os.path.join(GOLDEN, "m200_s1.prof"))
    s = F.SeqSet.concat([F.synth_sequences(4000, seed=95, lmax=3000), F.emit_homologs(p, 40, seed=96)])
    prof, db = api.DeviceProfile(ctx, p), api.DeviceDB(ctx, s)
    want = api.search(ctx, prof, db)
    out = torch.zeros(2 * db.n, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()
    torch.cuda.synchronize()
    assert _search_static(prof, db, out, stream.cuda_stream) == api.eslOK
    torch.cuda.synchronize()      # device-wide: stream-ordered pools give back what earlier calls freed
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert _search_static(prof, db, out, stream.cuda_stream) == api.eslOK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert np.array_equal(out.cpu().numpy(), np.concatenate(want))
    ctx.close()
