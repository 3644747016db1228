"""In-HBM qubit remap (hq_state_remap), the single-GPU form of the reference's
layout change (src/executor.cpp:59-179): a permutation of the physical bits
that moves more than one pair of bits runs as one out-of-place pass (every
amplitude read and written once), a single exchange in place.  Checked
bit-exactly against a numpy permutation of the loaded state: amplitudes are
moved, never computed."""
import ctypes as C

import numpy as np
import pytest

from hyquas_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def physical(hq, s):
    """The state's device array in physical order, copied as is."""
    import torch

    p = C.c_void_p()
    hq.check(hq.lib.hq_state_device_ptr(s.handle, C.byref(p)))
    hq.synchronize()

    class Dev:
        __cuda_array_interface__ = {"shape": (1 << s.n,), "typestr": "<c8",
                                    "data": (p.value, False), "version": 3}

    return torch.as_tensor(Dev(), device="cuda").cpu().numpy().copy()


def expected_physical(psi, pos):
    """Physical array whose bit pos[q] carries logical qubit q."""
    n = len(pos)
    out = np.empty_like(psi)
    idx = np.arange(psi.size, dtype=np.int64)
    phys = np.zeros_like(idx)
    for q in range(n):
        phys |= ((idx >> q) & 1) << pos[q]
    out[phys] = psi
    return out


@pytest.mark.parametrize("n,seed", [(7, 1), (12, 2), (20, 3)])
def test_remap_moves_every_amplitude(hq, n, seed):
    psi = W.random_state(seed, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    rng = W.SplitMix64(seed)
    for trial in range(4):
        pos = rng.shuffle(list(range(n)))
        if trial == 3:  # a single exchange takes the in-place path
            pos = list(range(n))
            pos[1], pos[n - 1] = pos[n - 1], pos[1]
        s.remap(pos)
        assert s.layout() == pos
        np.testing.assert_array_equal(physical(hq, s), expected_physical(psi, pos))
    s.remap(list(range(n)))
    np.testing.assert_array_equal(s.store(), psi)
    s.free()


def test_remap_full_reversal_26_qubits(hq):
    """Every bit moves (bit b to n-1-b): logical readout, norm and marginals are
    unchanged, and reversing again restores the physical array."""
    n = 26
    psi = W.random_state(11, n)
    s = hq.State(n, zero=False)
    s.load(psi)
    m0 = s.marginals()
    rev = list(range(n))[::-1]
    s.remap(rev)
    idx = np.array(W.SplitMix64(4).shuffle(range(1 << 16))[:4096], dtype=np.uint64) << np.uint64(10)
    np.testing.assert_array_equal(s.amps(idx), psi[idx.astype(np.int64)])
    np.testing.assert_allclose(s.marginals(), m0, rtol=0, atol=1e-9)
    s.remap(list(range(n)))
    np.testing.assert_array_equal(physical(hq, s), psi)
    s.free()
