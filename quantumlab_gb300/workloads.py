"""Seeded synthetic workloads: the five benchmark configurations as gate lists.

There is no public benchmark suite for this path; these generators restate the
configurations' shapes, sizes and value distributions.  All randomness comes
from one counter-free generator (splitmix64 seeding xoshiro256**, Box-Muller
for Gaussians) so the GPU runs, the oracle and the reference build see the
same gates.

Ops are tuples:
  ("cu", t, ar, ai, br, bi)   compactUnitary(t, alpha, beta)
  ("cx", c, t)                controlledNot(c, t)
  ("cp", a, b, theta)         controlledPhaseShift(a, b, theta)
  ("deph", t, p) / ("depol", t, p) / ("damp", t, p)   one-qubit channels
  ("h", t)                    hadamard(t)
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

import numpy as np

MASK64 = (1 << 64) - 1


class Xoshiro:
    """xoshiro256** seeded through splitmix64 (Blackman & Vigna)."""

    def __init__(self, seed: int):
        x = seed & MASK64
        s = []
        for _ in range(4):
            x = (x + 0x9E3779B97F4A7C15) & MASK64
            z = x
            z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
            z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
            s.append(z ^ (z >> 31))
        self.s = s

    @staticmethod
    def _rotl(x, k):
        return ((x << k) | (x >> (64 - k))) & MASK64

    def next(self) -> int:
        s = self.s
        result = (self._rotl((s[1] * 5) & MASK64, 7) * 9) & MASK64
        t = (s[1] << 17) & MASK64
        s[2] ^= s[0]
        s[3] ^= s[1]
        s[1] ^= s[2]
        s[0] ^= s[3]
        s[2] ^= t
        s[3] = self._rotl(s[3], 45)
        return result

    def uniform(self) -> float:
        """[0, 1) with 53 random bits."""
        return (self.next() >> 11) * (1.0 / (1 << 53))

    def uniform_open(self) -> float:
        """(0, 1]"""
        return 1.0 - self.uniform()

    def gauss(self) -> float:
        u1, u2 = self.uniform_open(), self.uniform()
        return math.sqrt(-2.0 * math.log(u1)) * math.cos(2.0 * math.pi * u2)

    def randint(self, n: int) -> int:
        return int(self.uniform() * n)

    def permutation(self, n: int) -> List[int]:
        p = list(range(n))
        for i in range(n - 1, 0, -1):
            j = self.randint(i + 1)
            p[i], p[j] = p[j], p[i]
        return p


def haar_pair(rng: Xoshiro) -> Tuple[float, float, float, float]:
    """(alpha, beta) from two normalised complex standard normals: a
    Haar-random SU(2) element in compactUnitary form."""
    g = [rng.gauss() for _ in range(4)]
    nrm = math.sqrt(sum(v * v for v in g))
    return g[0] / nrm, g[1] / nrm, g[2] / nrm, g[3] / nrm


def brickwork(n: int, layer: int) -> List[Tuple[int, int]]:
    """CNOT pairs (2i, 2i+1) on even layers, (2i+1, 2i+2) on odd layers."""
    if layer % 2 == 0:
        return [(2 * i, 2 * i + 1) for i in range(n // 2)]
    return [(2 * i + 1, 2 * i + 2) for i in range((n - 1) // 2)]


def c1_circuit(n: int = 20, layers: int = 40, seed: int = 1):
    """Plain FP64 random circuit: per layer a Haar compactUnitary on every
    qubit, then CNOT brickwork."""
    rng = Xoshiro(seed)
    ops = []
    for layer in range(layers):
        for q in range(n):
            ops.append(("cu", q) + haar_pair(rng))
        for c, t in brickwork(n, layer):
            ops.append(("cx", c, t))
    return ops


def c2_circuit(n: int = 30, layers: int = 20, seed: int = 2):
    """Per layer: Haar 1q on all qubits, controlledPhaseShift theta~U(0,2pi)
    on a random perfect matching, CNOT brickwork."""
    rng = Xoshiro(seed)
    ops = []
    for layer in range(layers):
        for q in range(n):
            ops.append(("cu", q) + haar_pair(rng))
        perm = rng.permutation(n)
        for i in range(n // 2):
            a, b = perm[2 * i], perm[2 * i + 1]
            ops.append(("cp", min(a, b), max(a, b), 2 * math.pi * rng.uniform()))
        for c, t in brickwork(n, layer):
            ops.append(("cx", c, t))
    return ops


def c3_circuit(nq: int = 14, layers: int = 10, seed: int = 3):
    """Noisy density matrix: Haar 1q + CNOT brickwork per layer, then on every
    qubit dephasing p~U(0,.05), depolarising p~U(0,.03), damping p~U(0,.02)."""
    rng = Xoshiro(seed)
    ops = []
    for layer in range(layers):
        for q in range(nq):
            ops.append(("cu", q) + haar_pair(rng))
        for c, t in brickwork(nq, layer):
            ops.append(("cx", c, t))
        for q in range(nq):
            ops.append(("deph", q, 0.05 * rng.uniform()))
            ops.append(("depol", q, 0.03 * rng.uniform()))
            ops.append(("damp", q, 0.02 * rng.uniform()))
    return ops


def algorithmic_bytes(ops, n: int, amp_bytes: int = 16) -> int:
    """Bytes a per-gate simulator must stream: 1q gate 2*2^n amps (r+w),
    CNOT 2*2^(n-1), CPhase 2*2^(n-2), DM channels per their touched entries."""
    N = 1 << n
    total = 0
    for op in ops:
        k = op[0]
        if k in ("cu", "h"):
            total += 2 * N * amp_bytes
        elif k == "cx":
            total += N * amp_bytes
        elif k == "cp":
            total += (N // 2) * amp_bytes
        elif k == "deph":
            total += N * amp_bytes
        elif k in ("depol", "damp"):
            total += 2 * N * amp_bytes
    return total


def run_ops(L, q, ops: Sequence[tuple], density_doubling: bool = True):
    """Issue a gate list through a QuEST-ABI library binding (QuESTLibrary)."""
    from .quest import Complex
    lib = L.lib
    for op in ops:
        k = op[0]
        if k == "cu":
            lib.compactUnitary(q, op[1], Complex(op[2], op[3]), Complex(op[4], op[5]))
        elif k == "cx":
            lib.controlledNot(q, op[1], op[2])
        elif k == "cp":
            lib.controlledPhaseShift(q, op[1], op[2], op[3])
        elif k == "h":
            lib.hadamard(q, op[1])
        elif k == "ps":
            lib.phaseShift(q, op[1], op[2])
        elif k == "rz":
            lib.rotateZ(q, op[1], op[2])
        elif k == "deph":
            lib.mixDephasing(q, op[1], op[2])
        elif k == "depol":
            lib.mixDepolarising(q, op[1], op[2])
        elif k == "damp":
            lib.mixDamping(q, op[1], op[2])
        else:
            raise ValueError(f"unknown op {k}")


# ---------------------------------------------------------------- Hubbard
def hubbard_terms(sites: int, U: float, t: float = 1.0):
    """1D Fermi-Hubbard, open boundary, Jordan-Wigner with interleaved
    ordering q = 2*i + spin.  Returns (codes[T, n], coeffs[T], constant).
    Hopping c_p^dag c_q + h.c. between q and q+2 (same spin) is
    (X_p Z X_q + Y_p Z Y_q)/2 with the Z on the orbital between them;
    n_up n_dn = (1 - Z_up - Z_dn + Z_up Z_dn)/4."""
    n = 2 * sites
    codes, coeffs = [], []
    const = 0.0
    for i in range(sites - 1):
        for s in range(2):
            p, r = 2 * i + s, 2 * (i + 1) + s
            for pa in (1, 2):                    # X..X and Y..Y
                c = [0] * n
                c[p] = pa
                c[r] = pa
                for m in range(p + 1, r):
                    c[m] = 3
                codes.append(c)
                coeffs.append(-t / 2.0)
    for i in range(sites):
        up, dn = 2 * i, 2 * i + 1
        c = [0] * n
        c[up] = 3
        c[dn] = 3
        codes.append(c)
        coeffs.append(U / 4.0)
        for q in (up, dn):
            c = [0] * n
            c[q] = 3
            codes.append(c)
            coeffs.append(-U / 4.0)
        const += U / 4.0
    return np.array(codes, dtype=np.int32), np.array(coeffs), const


def neel_index(sites: int) -> int:
    """Half-filled Neel state |up dn, dn up, ...>: site i holds spin i%2
    (an occupied orbital is qubit value 1)."""
    idx = 0
    for i in range(sites):
        q = 2 * i + (i % 2)
        idx |= 1 << q
    return idx


def lab_trotter_ops(codes, coeffs, dt: float, steps: int, ancilla: int):
    """The gate sequence QuantumLab's Pauli-Trotter builder emits for a
    first-order Trotter circuit (PauliProduct::OneStepGate,
    Circuit/Gates/PauliSimulate.cpp:30-80): per term, a basis change and a CNOT
    ladder that computes the parity of the term's qubits into an ancilla
    (X: H, CX; Y: P(-pi/2), H, CX; Z: CX), Rz(-2 dt c) on the ancilla, then the
    same gates inverted in reverse order.  With the ancilla in |0> this is
    exp(-i phi/2 P) on the system with phi = -2 dt c, i.e. multiRotatePauli(P,
    phi).  Ops: ("h", q), ("ps", q, theta), ("cx", c, t), ("rz", q, theta)."""
    ops = []
    for _ in range(steps):
        for code, c in zip(codes, coeffs):
            prep = []
            for i, pa in enumerate(code):
                if pa == 1:
                    prep += [("h", i), ("cx", i, ancilla)]
                elif pa == 2:
                    prep += [("ps", i, -math.pi / 2), ("h", i), ("cx", i, ancilla)]
                elif pa == 3:
                    prep += [("cx", i, ancilla)]
            if not prep:
                continue
            ops += prep
            ops.append(("rz", ancilla, -2.0 * dt * c))
            for op in reversed(prep):                   # the dagger: inverse gates, reversed
                ops.append(("ps", op[1], -op[2]) if op[0] == "ps" else op)
    return ops


def hubbard_instances(count: int = 64):
    """(U, dt, order) per instance: U in {2,4,8}, dt in {.1,.05,.01}, order 1/2."""
    out = []
    for i in range(count):
        U = (2.0, 4.0, 8.0)[i % 3]
        dt = (0.1, 0.05, 0.01)[(i // 3) % 3]
        order = 1 + ((i // 9) % 2)
        out.append((U, dt, order))
    return out


# ---------------------------------------------------------------- swap tests
def gaussian_mixture_vectors(count: int = 4096, components: int = 16, dmin: int = 4, dmax: int = 10, seed: int = 5):
    """QKMeans inputs: per vector a dimension exponent d ~ U{dmin..dmax}, a
    mixture component, and a unit-normalised real vector of length 2^d drawn
    around that component's mean.  Returns (d[], comp[], vectors[],
    centroids) with centroids[d][c] the normalised component means.  Seeded
    through xoshiro256** into numpy's PCG64 (vectorised draws)."""
    x = Xoshiro(seed)
    rng = np.random.Generator(np.random.PCG64(x.next()))
    ds = rng.integers(dmin, dmax + 1, size=count)
    comps = rng.integers(0, components, size=count)
    centroids = {}
    for d in range(dmin, dmax + 1):
        m = rng.standard_normal((components, 1 << d))
        centroids[d] = m / np.linalg.norm(m, axis=1, keepdims=True)
    vecs = []
    for d, c in zip(ds, comps):
        dim = 1 << int(d)
        v = centroids[int(d)][c] + 0.3 / math.sqrt(dim) * rng.standard_normal(dim)
        vecs.append(v / np.linalg.norm(v))
    return [int(d) for d in ds], [int(c) for c in comps], vecs, centroids


def swap_test_pool(vecs, centroids, dmin: int = 4, dmax: int = 10):
    """Concatenate data vectors and centroids into one pool and list the
    (vector, centroid) pairs of equal dimension: every vector against every
    centroid of its dimension.  Returns (pool, offsets, dimLog2, idxA, idxB)."""
    items = list(vecs)
    dims = [int(round(math.log2(len(v)))) for v in vecs]
    cent_index = {}
    for d in range(dmin, dmax + 1):
        for c, m in enumerate(centroids[d]):
            cent_index[(d, c)] = len(items)
            items.append(m)
            dims.append(d)
    offsets = np.zeros(len(items), dtype=np.int64)
    pos = 0
    for i, v in enumerate(items):
        offsets[i] = pos
        pos += len(v)
    pool = np.concatenate(items).astype(np.float64)
    ncent = len(centroids[dmin])
    idx_a, idx_b = [], []
    for i, v in enumerate(vecs):
        d = dims[i]
        for c in range(ncent):
            idx_a.append(i)
            idx_b.append(cent_index[(d, c)])
    return pool, offsets, np.array(dims, dtype=np.int32), np.array(idx_a, dtype=np.int32), np.array(idx_b, dtype=np.int32)


def swap_test_plain(L, q, u, v, d: int, prepared: bool = False) -> float:
    """One swap test through the QuEST API, one kernel per gate (the
    reference pattern): initStateFromAmps(|0>|v>|u>) with u on qubits 0..d-1,
    v on d..2d-1, ancilla 2d; H; d controlled swaps as CNOT(v_i -> u_i),
    Toffoli(anc, u_i -> v_i), CNOT(v_i -> u_i); H; P(anc = 0).  `q` is a
    (2d+1)-qubit register that is reused between calls; with prepared=True it
    already holds |0>|v>|u>."""
    n = 2 * d + 1
    if not prepared:
        psi = np.zeros(1 << n, dtype=np.complex128)
        psi[: 1 << (2 * d)] = np.kron(v, u)
        L.set_amps(q, psi)
    anc = 2 * d
    L.lib.hadamard(q, anc)
    for i in range(d):
        a, b = i, d + i
        L.lib.controlledNot(q, b, a)
        L.multiControlledMultiQubitNot(q, [anc, a], [b])
        L.lib.controlledNot(q, b, a)
    L.lib.hadamard(q, anc)
    return L.lib.calcProbOfOutcome(q, anc, 0)
