"""The allocation-free marginals entry point (hq_marginals_noalloc).

It serves callers that cannot call cudaMalloc -- device memory owned by another
allocator, or paths that must not take cudaMalloc's implicit synchronisation --
so it uses a static device scratch array instead of allocating.  Checked
through the C ABI against the allocating entry point (hq_state_marginals /
hq_state_norm) on calls in a row, each smaller than the one before so it
runs over the earlier calls' leftover scratch contents, down to 1 and 3 qubits
where one reduction block sees mostly padding.  The caller's device
buffers here come from torch, standing in for the caller's own allocator."""
import ctypes as C

import numpy as np
import pytest

from hyquas_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _entry(hq):
    f = hq.lib.hq_marginals_noalloc
    f.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]
    f.restype = C.c_int32
    return f


def _dev_ptr(hq, state):
    p = C.c_void_p()
    hq.check(hq.lib.hq_state_device_ptr(state.handle, C.byref(p)))
    return p


def test_noalloc_marginals_match_allocating_entry_point(hq):
    import torch

    f = _entry(hq)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for seed, n in ((1, 26), (2, 19), (3, 3), (4, 1)):
        s = hq.State(n, zero=False)
        s.load(W.random_state(seed, n))
        out = torch.full((n + 1,), float("nan"), dtype=torch.float64, device="cuda")
        rc = f(_dev_ptr(hq, s), n, C.c_void_p(out.data_ptr()), stream)
        assert rc == 0, hq.lib.hq_last_error()
        got = out.cpu().numpy()  # ordered after the call on the same stream
        assert abs(got[0] - s.norm()) < 1e-9
        np.testing.assert_allclose(got[1:], s.marginals(), rtol=0, atol=1e-9)
        s.free()


def test_noalloc_marginals_rejects_sizes_beyond_its_scratch(hq):
    f = _entry(hq)
    rc = f(C.c_void_p(256), 27, C.c_void_p(256), None)
    assert rc == -1
    assert b"allocation-free range" in hq.lib.hq_last_error()
    assert f(None, 10, C.c_void_p(256), None) == -1


def test_noalloc_marginals_allocate_no_device_memory(hq):
    """After a first call (which looks up the scratch address), further calls
    leave the device's free memory unchanged."""
    import torch

    f = _entry(hq)
    n = 22
    s = hq.State(n, zero=False)
    s.load(W.random_state(5, n))
    out = torch.empty((n + 1,), dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert f(_dev_ptr(hq, s), n, C.c_void_p(out.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        assert f(_dev_ptr(hq, s), n, C.c_void_p(out.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 >= free0, (free0, free1)
    s.free()
