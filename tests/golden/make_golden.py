"""Generate the golden fixtures from the reference's own QuEST CPU build.

Run here, where the reference sources are mounted (they are not on the GPU
host):

    make -C oracle ref            # -> oracle/_ref/libquest_ref.so
    python tests/golden/make_golden.py

Writes, next to this script:
  api_cases.json.gz every catalogue case (ops + op results + probe results)
  api_amps.npz     final amplitudes per case
  circuits.npz     reduced-size versions of the benchmark workloads (the plain
                   random circuit, the noisy density matrix, a Fermi-Hubbard
                   Trotter run and swap tests): amplitudes/summaries
The reference library is only ever executed by this script.
"""
from __future__ import annotations

import gzip
import json
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from quantumlab_gb300.quest import QuESTLibrary  # noqa: E402
from quantumlab_gb300 import workloads as W     # noqa: E402
import quest_cases as QC                         # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref", "libquest_ref.so")


def circuit_goldens(L):
    out = {}
    # plain random circuit (benchmark config 1 structure), 12 qubits, 8 layers
    ops = W.c1_circuit(n=12, layers=8, seed=11)
    q = L.create(12)
    W.run_ops(L, q, ops)
    out["c1_amps"] = L.amps(q).copy()
    out["c1_total"] = np.array([L.lib.calcTotalProb(q)])
    out["c1_p1"] = np.array([L.lib.calcProbOfOutcome(q, t, 1) for t in range(12)])
    L.destroy(q)
    # random circuit with CPhase matchings (config 2 structure), 10 qubits, 6 layers
    ops = W.c2_circuit(n=10, layers=6, seed=12)
    q = L.create(10)
    W.run_ops(L, q, ops)
    out["c2_amps"] = L.amps(q).copy()
    L.destroy(q)
    # noisy density matrix (config 3 structure), 5 qubits, 4 layers
    ops = W.c3_circuit(nq=5, layers=4, seed=13)
    d = L.create(5, True)
    W.run_ops(L, d, ops)
    out["c3_amps"] = L.amps(d).copy()
    out["c3_trace"] = np.array([L.lib.calcTotalProb(d)])
    out["c3_purity"] = np.array([L.lib.calcPurity(d)])
    out["c3_p1"] = np.array([L.lib.calcProbOfOutcome(d, t, 1) for t in range(5)])
    L.destroy(d)
    # Fermi-Hubbard Trotter (config 4 structure), 4 sites = 8 qubits
    energies, occs = [], []
    for (U, dt, order) in [(2.0, 0.1, 1), (4.0, 0.05, 2), (8.0, 0.1, 2)]:
        codes, coeffs, const = W.hubbard_terms(4, U)
        q = L.create(8)
        L.lib.initClassicalState(q, W.neel_index(4))
        h = L.pauli_hamil(codes, coeffs)
        steps = int(round(1.0 / dt))
        L.lib.applyTrotterCircuit(q, h, 1.0, order, steps)
        ws = L.create(8)
        energies.append(L.calcExpecPauliSum(q, codes, coeffs, ws) + const)
        occs.append([L.lib.calcProbOfOutcome(q, t, 1) for t in range(8)])
        L.destroy(ws)
        L.lib.destroyPauliHamil(h)
        L.destroy(q)
    out["c4_energy"] = np.array(energies)
    out["c4_occ"] = np.array(occs)
    # swap tests (config 5 structure): |0>|u>|v>, H, d cswaps, H -> P(anc=0)
    p0s = []
    rng = QC.R(15)
    for d in (2, 3, 4):
        u = np.array([rng.g() for _ in range(1 << d)]); u /= np.linalg.norm(u)
        v = np.array([rng.g() for _ in range(1 << d)]); v /= np.linalg.norm(v)
        n = 2 * d + 1
        q = L.create(n)
        psi = np.kron(v, np.kron(u, np.array([1.0, 0.0])))   # anc = qubit 0, u = 1..d, v = d+1..2d
        L.set_amps(q, psi.astype(np.complex128))
        L.lib.hadamard(q, 0)
        for i in range(d):
            # controlled swap(anc; u_i, v_i) = CX(v,u) Toffoli(anc,u; v) CX(v,u)
            a, b = 1 + i, 1 + d + i
            L.lib.controlledNot(q, b, a)
            L.multiControlledUnitary(q, [0, a], b, np.array([[0, 1], [1, 0]]))
            L.lib.controlledNot(q, b, a)
        L.lib.hadamard(q, 0)
        p0s.append(L.lib.calcProbOfOutcome(q, 0, 0))
        L.destroy(q)
    out["c5_p0"] = np.array(p0s)
    return out


def main():
    if not os.path.exists(REF):
        raise SystemExit(f"{REF} missing: run `make -C oracle ref` where the reference is mounted")
    L = QuESTLibrary(REF)
    cases = QC.build_cases()
    amps = {}
    for i, c in enumerate(cases):
        a, results, probes = QC.run_case(L, c)
        c["results"] = results
        c["probe_values"] = probes
        amps[f"case{i}"] = a
    with gzip.open(os.path.join(HERE, "api_cases.json.gz"), "wt") as f:
        json.dump(cases, f)
    np.savez_compressed(os.path.join(HERE, "api_amps.npz"), **amps)
    np.savez_compressed(os.path.join(HERE, "circuits.npz"), **circuit_goldens(L))
    print(f"{len(cases)} cases written")


if __name__ == "__main__":
    main()
