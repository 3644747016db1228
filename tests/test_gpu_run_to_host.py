"""hq_circuit_run_to_host: a run followed by the full-state readback of the
reference's Circuit::run + result (src/circuit.cpp:46-62).  The fused form
(the last group writes HBM and the pinned host buffer in one pass) must give
exactly the bytes of run + store; the copy form covers unpinned buffers and
runs that end outside the canonical layout."""
import numpy as np
import pytest

from hyquas_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _compiled(hq, n, desc):
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile("oshm", specialize=1)  # generated kernels for every group
    return c


def _run_and_store(hq, c, n):
    s = hq.State(n)
    s.init_zero()
    c.run_on(s)
    return s.store()


def test_fused_readback_is_run_then_store(hq, oracle):
    n = 24  # 128 MiB: the huge-page pinned buffer path
    desc = W.grid_random(5, 2, 12, 6)
    c = _compiled(hq, n, desc)
    ref = _run_and_store(hq, c, n)
    buf = hq.PinnedBuffer(1 << n)
    buf.array[:] = np.complex64(complex(np.nan, np.nan))
    s = hq.State(n)
    s.init_zero()
    us = c.run_to_host(s, buf.array)
    assert us > 0
    assert np.array_equal(buf.array, ref)  # every amplitude written, bit for bit
    assert np.array_equal(s.store(), ref)  # and the device state holds the same
    cmp = oracle.compare(oracle.run_f64(n, desc), buf.array)
    assert cmp["max_abs_err"] <= 1e-5 and cmp["one_minus_fidelity"] <= 1e-6, cmp


def test_unpinned_buffer_takes_the_copy(hq):
    n = 20
    desc = W.grid_random(6, 4, 5, 5)
    c = _compiled(hq, n, desc)
    ref = _run_and_store(hq, c, n)
    out = np.full(1 << n, np.nan, dtype=np.complex64)
    s = hq.State(n)
    s.init_zero()
    c.run_to_host(s, out)
    assert np.array_equal(out, ref)


def test_run_ending_in_a_swapped_layout_reads_back_logical_order(hq, oracle):
    n = 18
    desc = W.grid_random(7, 3, 6, 4) + [(W.SWAP, 0, 17, -1, ()), (W.SWAP, 3, 12, -1, ())]
    c = _compiled(hq, n, desc)
    buf = hq.PinnedBuffer(1 << n)
    s = hq.State(n)
    s.init_zero()
    c.run_to_host(s, buf.array)
    cmp = oracle.compare(oracle.run_f64(n, desc), buf.array)
    assert cmp["max_abs_err"] <= 1e-5 and cmp["one_minus_fidelity"] <= 1e-6, cmp
    assert np.array_equal(s.store(), buf.array)


def test_run_to_host_rejects_a_wrong_buffer(hq):
    n = 10
    c = _compiled(hq, n, W.grid_random(8, 2, 5, 2))
    s = hq.State(n)
    s.init_zero()
    with pytest.raises(ValueError):
        c.run_to_host(s, np.zeros(1 << (n - 1), dtype=np.complex64))


def test_async_readback_beside_the_next_run(hq):
    """State.store_async into a large pinned buffer runs as a copy kernel on a
    few SMs; a circuit run on another state meanwhile launches its persistent
    kernels on the other SMs.  Both results are exact."""
    n = 24
    ca = _compiled(hq, n, W.grid_random(9, 2, 12, 5))
    cb = _compiled(hq, n, W.grid_random(10, 2, 12, 5))
    ref_a = _run_and_store(hq, ca, n)
    ref_b = _run_and_store(hq, cb, n)
    sa, sb = hq.State(n), hq.State(n)
    buf = hq.PinnedBuffer(1 << n)
    buf.array[:] = np.complex64(complex(np.nan, np.nan))
    sa.init_zero()
    ca.run_on(sa)
    sa.store_async(buf.array)
    sb.init_zero()
    cb.run_on(sb)
    sa.wait()
    assert np.array_equal(buf.array, ref_a)
    assert np.array_equal(sb.store(), ref_b)


def test_run_to_host_after_a_transmm_group(hq, oracle):
    """A schedule whose last group is a TransMM group reads back by copy."""
    n = 21
    desc = W.blocked_u3_cnot(12, n, 7, 6, 1)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile("transmm")
    assert all(b == hq.BACKEND_TRANSMM for (b, _, _, _) in c.schedule())
    buf = hq.PinnedBuffer(1 << n)
    s = hq.State(n)
    s.init_zero()
    c.run_to_host(s, buf.array)
    cmp = oracle.compare(oracle.run_f64(n, desc), buf.array)
    assert cmp["max_abs_err"] <= 1e-5 and cmp["one_minus_fidelity"] <= 1e-6, cmp


@pytest.mark.parametrize("n,pinned", [(20, True), (20, False), (23, True)])
def test_async_readback_small_and_unpinned_buffers(hq, n, pinned):
    """Below 64 MiB, or into pageable memory, store_async copies with the copy
    engine; from 64 MiB of pinned memory up, with the copy kernel.  All give
    the bytes of a synchronous store."""
    c = _compiled(hq, n, W.grid_random(13, 4, n // 4, 4) if n % 4 == 0 else W.grid_random(13, 1, n, 4))
    ref = _run_and_store(hq, c, n)
    s = hq.State(n)
    s.init_zero()
    c.run_on(s)
    buf = hq.PinnedBuffer(1 << n) if pinned else None
    out = buf.array if pinned else np.empty(1 << n, dtype=np.complex64)
    out[:] = np.complex64(complex(np.nan, np.nan))
    s.store_async(out)
    s.wait()
    assert np.array_equal(out, ref)
