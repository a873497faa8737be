"""QuantumLab's Pauli-Trotter builder through the QuEST API (GPU).

The lab expands every Pauli term into a basis change, a CNOT ladder into an
ancilla, an ancilla Rz and the inverse (PauliProduct::OneStepGate,
Circuit/Gates/PauliSimulate.cpp:30-80).  Issued gate by gate, that sequence
must equal multiRotatePauli per term on the system qubits, with the ancilla
back in |0>: exactly in FP64, and to the fused engine's bounds with op-stream
capture on (which turns every term's ladder into at most one fused pass)."""
import numpy as np
import pytest

from quantumlab_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def no_library_errors(gpulib):
    gpulib.capture_errors()
    gpulib.errors.clear()
    yield
    errors = list(gpulib.errors)
    gpulib.errors.clear()
    assert not errors, errors


def reference_state(L, codes, coeffs, dt, steps, n, start):
    q = L.create(n)
    L.lib.initClassicalState(q, start)
    for _ in range(steps):
        for code, c in zip(codes, coeffs):
            targets = [i for i, p in enumerate(code) if p]
            if targets:
                L.multiRotatePauli(q, targets, [int(code[i]) for i in targets], -2.0 * dt * c)
    a = L.amps(q).copy()
    L.destroy(q)
    return a


@pytest.mark.parametrize("capture", [0, 1])
def test_lab_trotter_expansion_equals_multi_rotate_pauli(gpulib, capture):
    L = gpulib
    sites = 5
    codes, coeffs, _ = W.hubbard_terms(sites, 4.0)
    nsys = 2 * sites
    n = nsys + 1                                        # the ancilla is the top qubit
    dt, steps = 0.1, 3
    start = W.neel_index(sites)
    want = reference_state(L, codes, coeffs, dt, steps, n, start)
    ops = W.lab_trotter_ops(codes, coeffs, dt, steps, ancilla=nsys)
    q = L.create(n)
    L.lib.quest_gb300_setCapture(q, capture)
    L.lib.initClassicalState(q, start)
    W.run_ops(L, q, ops)
    got = L.amps(q)
    err = np.max(np.abs(got - want))
    anc = np.sum(np.abs(got[1 << nsys:]) ** 2)          # probability of the ancilla in |1>
    print(f"capture={capture}: {len(ops)} gates, max|d amp| {err:.2e}, P(anc=1) {anc:.1e}")
    if capture:
        assert err < 1e-5 and anc < 1e-9
    else:
        assert err < 1e-12 and anc < 1e-24
    L.destroy(q)
