"""The reference's own single-GPU runs replayed on the GB300 (oracle/ref_replay.cu):
its kernels (src/kernelOpt.cu run<128>, src/kernelSimple.cu), compiled from
its sources for sm_103a, launched with the arguments its host code produced.
The replayed states must match the FP64 oracle like this library's own paths
do, which shows the replay is the reference's computation and makes its timing
in bench.py a like-for-like baseline."""
import numpy as np
import pytest

from hyquas_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-5
FID = 1e-6


def _circuit(O, name):
    import importlib.util
    from pathlib import Path
    spec = importlib.util.spec_from_file_location(
        "hq_make_ref_traces", Path(O.__file__).resolve().parent / "make_ref_traces.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.circuits()[name]


@pytest.mark.parametrize("name", ["grid16_group", "mixed14_group", "mixed14_serial"])
def test_reference_replay_matches_oracle(hq, oracle, name):
    if not oracle.ref_gpu_available(name):
        pytest.skip("traces are built where the reference checkout is present")
    n, desc, backend = _circuit(oracle, name)
    r = oracle.ref_gpu_run(name, repeats=1)
    assert r["num_qubits"] == n
    c = oracle.compare(oracle.run_f64(n, desc), r["state"])
    assert c["max_abs_err"] <= TOL and c["one_minus_fidelity"] <= FID, c
    if backend == "serial":
        assert r["launches"] == len(desc)
    else:
        assert r["launches"] == r["groups"]


def test_reference_replay_agrees_with_this_library(hq, oracle):
    """Same circuit, the reference's OShareMem kernel and this library's
    generated kernels: the two complex64 states agree."""
    name = "grid16_group"
    if not oracle.ref_gpu_available(name):
        pytest.skip("traces are built where the reference checkout is present")
    n, desc, _ = _circuit(oracle, name)
    r = oracle.ref_gpu_run(name, repeats=1)
    c = hq.Circuit(n)
    c.addGates(W.to_gates(desc))
    c.compile("oshm")
    s = hq.State(n)
    c.run_on(s)
    ours = s.store()
    assert np.max(np.abs(ours.astype(np.complex128) - r["state"])) <= 2 * TOL
