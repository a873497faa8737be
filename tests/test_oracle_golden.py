"""The oracle (CPU restatement) against the reference's own outputs.

tests/golden/* were produced by the reference's QuEST CPU build
(tests/golden/make_golden.py); this pins the oracle before it is trusted as
the checker of the GPU library."""
import numpy as np
import pytest

import quest_cases as QC
from parity import check_case
from quantumlab_gb300 import workloads as W


def test_catalogue_against_reference(oracle, golden):
    cases, amps, _ = golden
    assert len(cases) > 700
    for i, case in enumerate(cases):
        a, results, probes = QC.run_case(oracle, case)
        check_case(case, a, results, probes, amps[f"case{i}"])


def test_circuits_against_reference(oracle, golden):
    _, _, circ = golden
    L = oracle
    q = L.create(12)
    W.run_ops(L, q, W.c1_circuit(n=12, layers=8, seed=11))
    assert np.max(np.abs(L.amps(q) - circ["c1_amps"])) < 1e-12
    assert abs(L.lib.calcTotalProb(q) - circ["c1_total"][0]) < 1e-12
    L.destroy(q)
    q = L.create(10)
    W.run_ops(L, q, W.c2_circuit(n=10, layers=6, seed=12))
    assert np.max(np.abs(L.amps(q) - circ["c2_amps"])) < 1e-12
    L.destroy(q)
    d = L.create(5, True)
    W.run_ops(L, d, W.c3_circuit(nq=5, layers=4, seed=13))
    assert np.max(np.abs(L.amps(d) - circ["c3_amps"])) < 1e-12
    assert abs(L.lib.calcPurity(d) - circ["c3_purity"][0]) < 1e-12
    L.destroy(d)


def test_swap_test_closed_form(golden):
    """P(anc=0) of the reference swap test matches (1 + |<u|v>|^2)/2."""
    _, _, circ = golden
    rng = QC.R(15)
    for d, p0 in zip((2, 3, 4), circ["c5_p0"]):
        u = np.array([rng.g() for _ in range(1 << d)]); u /= np.linalg.norm(u)
        v = np.array([rng.g() for _ in range(1 << d)]); v /= np.linalg.norm(v)
        assert abs(p0 - (1 + np.dot(u, v) ** 2) / 2) < 1e-12


def test_hubbard_energy_conserved_small_dt(golden):
    """Trotter energies stay near the Neel start energy (Neel is an
    eigenstate of the interaction part only; sanity bounds)."""
    _, _, circ = golden
    assert np.all(np.isfinite(circ["c4_energy"]))
    assert np.allclose(circ["c4_occ"].sum(axis=1), 4.0, atol=1e-9)   # particle number 4 of 8 orbitals
