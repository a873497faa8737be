"""The gate-fusion planner (host code, no GPU): the product of a compiled
plan's pass matrices must reproduce the circuit exactly (FP64), and passes
respect the fusion width."""
import ctypes as C

import numpy as np
import pytest

import quantumlab_gb300 as qg
from quantumlab_gb300 import workloads as W


@pytest.fixture(scope="module")
def lib():
    path = qg.build()
    L = C.CDLL(path, mode=C.RTLD_LOCAL)
    L.quest_gb300_planCreate.restype = C.c_void_p
    L.quest_gb300_planCreate.argtypes = [C.c_int, C.c_int]
    L.quest_gb300_planDestroy.argtypes = [C.c_void_p]
    L.quest_gb300_planAddCompactUnitary.argtypes = [C.c_void_p, C.c_int] + [C.c_double] * 4
    L.quest_gb300_planAddControlledNot.argtypes = [C.c_void_p, C.c_int, C.c_int]
    L.quest_gb300_planAddControlledPhaseShift.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_double]
    L.quest_gb300_planAddHadamard.argtypes = [C.c_void_p, C.c_int]
    L.quest_gb300_planAddGate.argtypes = [C.c_void_p, C.POINTER(C.c_int), C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.quest_gb300_planSetBeamWidth.argtypes = [C.c_void_p, C.c_int]
    L.quest_gb300_planCompile.argtypes = [C.c_void_p]
    L.quest_gb300_planPass.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.quest_gb300_planSetMaxControls.argtypes = [C.c_void_p, C.c_int]
    L.quest_gb300_planSetLookahead.argtypes = [C.c_void_p, C.c_int]
    L.quest_gb300_planPassControls.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int)]
    L.quest_gb300_planPassBlock.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    return L


def make_plan(L, n, kmax, ops, beam=None, controls=None, lookahead=None):
    """Compile; returns [(targets, matrix)], or with `controls` (the plan's
    control limit) [(targets, control qubits, [matrix per control value])]."""
    p = L.quest_gb300_planCreate(n, kmax)
    if beam is not None:
        assert L.quest_gb300_planSetBeamWidth(p, beam) == 0
    if lookahead is not None:
        assert L.quest_gb300_planSetLookahead(p, lookahead) == 0
    assert L.quest_gb300_planSetMaxControls(p, controls or 0) == 0
    for op in ops:
        if op[0] == "m":                          # ("m", qubits, matrix)
            re = np.ascontiguousarray(op[2].real.ravel())
            im = np.ascontiguousarray(op[2].imag.ravel())
            assert L.quest_gb300_planAddGate(p, (C.c_int * len(op[1]))(*op[1]), len(op[1]),
                                             re.ctypes.data_as(C.POINTER(C.c_double)),
                                             im.ctypes.data_as(C.POINTER(C.c_double))) == 0
        elif op[0] == "cu":
            assert L.quest_gb300_planAddCompactUnitary(p, *op[1:]) == 0
        elif op[0] == "cx":
            assert L.quest_gb300_planAddControlledNot(p, op[1], op[2]) == 0
        elif op[0] == "cp":
            assert L.quest_gb300_planAddControlledPhaseShift(p, op[1], op[2], op[3]) == 0
    npass = L.quest_gb300_planCompile(p)
    passes = []
    for i in range(npass):
        t = (C.c_int * 6)()
        re = np.zeros(4096)
        im = np.zeros(4096)
        k = L.quest_gb300_planPass(p, i, t, re.ctypes.data_as(C.POINTER(C.c_double)), im.ctypes.data_as(C.POINTER(C.c_double)))
        D = 1 << k
        if controls is None:
            passes.append((list(t[:k]), (re[:D * D] + 1j * im[:D * D]).reshape(D, D)))
            continue
        cq = (C.c_int * 3)()
        nc = L.quest_gb300_planPassControls(p, i, cq)
        blocks = []
        for b in range(1 << nc):
            assert L.quest_gb300_planPassBlock(p, i, b, re.ctypes.data_as(C.POINTER(C.c_double)),
                                               im.ctypes.data_as(C.POINTER(C.c_double))) == k
            blocks.append((re[:D * D] + 1j * im[:D * D]).reshape(D, D))
        passes.append((list(t[:k]), list(cq[:nc]), blocks))
    L.quest_gb300_planDestroy(p)
    return passes


def apply_matrix(psi, n, targets, m):
    """apply m (matrix bit b on targets[b]) to psi (index bit q = qubit q)"""
    k = len(targets)
    t = psi.reshape([2] * n)                   # axis a <-> qubit n-1-a
    axes = [n - 1 - q for q in reversed(targets)]   # matrix row index bits high..low
    t = np.moveaxis(t, axes, list(range(k)))
    shp = t.shape
    t = (m @ t.reshape(1 << k, -1)).reshape(shp)
    t = np.moveaxis(t, list(range(k)), axes)
    return t.reshape(-1)


def reference(n, ops):
    psi = np.zeros(1 << n, dtype=complex)
    psi[0] = 1
    return reference_from(psi, n, ops)


def reference_from(psi, n, ops):
    for op in ops:
        if op[0] == "cu":
            a, b = complex(op[2], op[3]), complex(op[4], op[5])
            psi = apply_matrix(psi, n, [op[1]], np.array([[a, -b.conjugate()], [b, a.conjugate()]]))
        elif op[0] == "cx":
            m = np.eye(4)[[0, 3, 2, 1]]
            psi = apply_matrix(psi, n, [op[1], op[2]], m)
        elif op[0] == "cp":
            psi = apply_matrix(psi, n, [op[1], op[2]], np.diag([1, 1, 1, np.exp(1j * op[3])]))
        elif op[0] == "m":
            psi = apply_matrix(psi, n, list(op[1]), op[2])
    return psi


def haar(rng, k):
    z = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
    return np.linalg.qr(z)[0]


def controlled(u, nc):
    """controls on matrix bits 0..nc-1, u on the bits above"""
    D = len(u) << nc
    m = np.eye(D, dtype=complex)
    on = (1 << nc) - 1
    rows = [r for r in range(D) if r & on == on]
    m[np.ix_(rows, rows)] = u
    return m


def mixed_ops(n, count, seed):
    """Dense, diagonal and controlled gates on 1-5 qubits: the planner's
    commutation rule meets every case (diagonal on all, some or none of a
    gate's qubits)."""
    rng = np.random.default_rng(seed)
    ops = []
    for _ in range(count):
        kind = rng.integers(5)
        k = int(rng.integers(1, 6)) if kind < 2 else int(rng.integers(2, 5))
        qs = [int(x) for x in rng.choice(n, size=k, replace=False)]
        if kind == 0:
            m = haar(rng, k)
        elif kind == 1:
            m = np.diag(np.exp(1j * rng.uniform(0, 2 * np.pi, size=1 << k)))
        elif kind == 2:
            nc = int(rng.integers(1, k))
            m = controlled(haar(rng, k - nc), nc)
        elif kind == 3:                            # controlled diagonal on a target: diagonal everywhere
            m = controlled(np.diag(np.exp(1j * rng.uniform(0, 2 * np.pi, size=1 << (k - 1)))), 1)
        else:                                      # CNOT-like permutation with one control
            perm = np.eye(1 << (k - 1))[rng.permutation(1 << (k - 1))]
            m = controlled(perm.astype(complex), 1)
        ops.append(("m", qs, m))
    return ops


@pytest.mark.parametrize("kmax", [1, 2, 3, 4, 5, 6])
def test_plan_reproduces_circuit(lib, kmax):
    n = 9
    ops = W.c2_circuit(n=n, layers=5, seed=3)
    if kmax == 1:
        ops = [o for o in ops if o[0] == "cu"]
    passes = make_plan(lib, n, kmax, ops)
    assert all(len(t) <= kmax for t, _ in passes)
    assert all(t == sorted(t) for t, _ in passes)
    psi = np.zeros(1 << n, dtype=complex)
    psi[0] = 1
    for t, m in passes:
        psi = apply_matrix(psi, n, t, m)
    ref = reference(n, ops)
    assert np.max(np.abs(psi - ref)) < 1e-12
    for _, m in passes:
        assert np.allclose(m @ m.conj().T, np.eye(len(m)), atol=1e-12)


@pytest.mark.parametrize("kmax,beam,seed", [(5, 8, 1), (6, 8, 2), (6, 1, 3), (6, 32, 4), (4, 4, 5)])
def test_plan_reproduces_mixed_circuit(lib, kmax, beam, seed):
    n = 9
    ops = mixed_ops(n, 60, seed)
    ops = [o for o in ops if len(o[1]) <= kmax]
    passes = make_plan(lib, n, kmax, ops, beam)
    assert all(len(t) <= kmax and t == sorted(t) for t, _ in passes)
    rng = np.random.default_rng(seed)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    want = psi.copy()
    for op in ops:
        want = apply_matrix(want, n, list(op[1]), op[2])
    for t, m in passes:
        psi = apply_matrix(psi, n, t, m)
    assert np.max(np.abs(psi - want)) < 1e-12


def test_plan_pass_count_30q(lib):
    ops = W.c2_circuit(n=30, layers=20, seed=2)
    counts = {k: len(make_plan(lib, 30, k, ops)) for k in (4, 5, 6)}
    # plain per-gate execution would need 1190 passes; merging gates into
    # open blocks in program order took 205, 168 and 130
    assert counts[4] <= 190 and counts[5] <= 140 and counts[6] <= 105, counts
    assert counts[6] <= counts[5] <= counts[4]


def test_plan_pass_count_brickwork(lib):
    ops = W.c1_circuit(n=20, layers=40, seed=1)
    # 1180 gates; merging in program order took 85 passes
    assert len(make_plan(lib, 20, 6, ops)) <= 45


def apply_controlled(psi, n, targets, controls, blocks):
    """block c acts on the amplitudes whose control bits are c (bit j <->
    controls[j]); it moves amplitudes only across target bits"""
    idx = np.arange(1 << n)
    val = np.zeros(1 << n, dtype=np.int64)
    for j, q in enumerate(controls):
        val |= ((idx >> q) & 1) << j
    out = np.zeros_like(psi)
    for c, m in enumerate(blocks):
        sel = val == c
        out[sel] = apply_matrix(psi, n, targets, m)[sel]
    return out


@pytest.mark.parametrize("kmax,maxctl,kind", [(6, 3, "c2"), (6, 1, "c2"), (5, 2, "c2"), (4, 3, "c2"),
                                              (6, 3, "mixed"), (5, 3, "mixed")])
def test_controlled_passes_reproduce_circuit(lib, kmax, maxctl, kind):
    """Passes with control qubits: gates diagonal on qubits outside a pass's
    targets (above its tile) are absorbed with those qubits as controls, and
    the pass applies the product of control value c to the amplitudes whose
    control bits are c.  Applied that way, the plan reproduces the circuit
    exactly; control qubits lie outside the targets and have at least 7
    non-target qubits below them; the plan needs fewer passes."""
    n = 15
    if kind == "c2":
        ops = W.c2_circuit(n=n, layers=8, seed=11)
    else:
        ops = [o for o in mixed_ops(n, 120, 7) if len(o[1]) <= kmax]
    passes = make_plan(lib, n, kmax, ops, controls=maxctl)
    plain = make_plan(lib, n, kmax, ops, controls=0)
    rng = np.random.default_rng(5)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    want = psi.copy()
    if kind == "c2":
        want = reference_from(psi, n, ops)
    else:
        for op in ops:
            want = apply_matrix(want, n, list(op[1]), op[2])
    used = 0
    for t, cs, blocks in passes:
        assert len(cs) <= maxctl and not set(cs) & set(t) and len(blocks) == 1 << len(cs)
        for c in cs:
            assert c - sum(1 for q in t if q < c) >= 7
        if cs:
            assert len(t) >= 4
        used += len(cs) > 0
        psi = apply_controlled(psi, n, t, cs, blocks)
    assert np.max(np.abs(psi - want)) < 1e-12
    assert used > 0 and len(passes) <= len(plain)
    print(f"{kind} k<={kmax} controls<={maxctl}: {len(passes)} passes ({used} controlled) against {len(plain)}")


def test_controlled_pass_count_30q(lib):
    """The 30-qubit, 20-layer random circuit at k <= 6: with up to three
    control qubits per pass the controlled phases of the random matching no
    longer need both qubits in one pass (101 passes without controls)."""
    ops = W.c2_circuit(n=30, layers=20, seed=2)
    counts = {m: len(make_plan(lib, 30, 6, ops, controls=m)) for m in (0, 1, 3)}
    assert counts[0] <= 105 and counts[1] <= 86 and counts[3] <= 68, counts
    assert counts[3] < counts[1] < counts[0]


def pauli_rotation(row, angle):
    """exp(-i angle/2 P) for the Pauli string `row` (0..3 per qubit) on its
    non-identity qubits (matrix bit b <-> the b-th of them)"""
    paulis = [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.diag([1, -1])]
    qs = [q for q, c in enumerate(row) if c]
    m = np.array([[1.0 + 0j]])
    for q in reversed(qs):
        m = np.kron(m, paulis[row[q]])
    return qs, np.cos(angle / 2) * np.eye(len(m)) - 1j * np.sin(angle / 2) * m


def test_lookahead_pass_counts(lib):
    """The search's lookahead: the best candidate sets tried one pass ahead.
    30-qubit random circuit with up to three control qubits: 65 passes
    without it, at most 64 with 4 candidates and 63 with 8; first-order
    Fermi-Hubbard Trotter circuit (24 qubits, 10 steps): 58 without, at most
    52 with 4.  Both plans still reproduce their circuits (the products are
    checked by the other tests)."""
    ops = W.c2_circuit(n=30, layers=20, seed=2)
    counts = {la: len(make_plan(lib, 30, 6, ops, controls=3, lookahead=la)) for la in (0, 4, 8)}
    assert counts[0] <= 66 and counts[4] <= 64 and counts[8] <= 63 and counts[8] <= counts[4] <= counts[0], counts
    codes, coeffs, _ = W.hubbard_terms(12, 4.0)
    hub = []
    for _ in range(10):
        for row, c in zip(codes, coeffs):
            qs, m = pauli_rotation([int(x) for x in row], 2 * c * 0.1)
            if qs:
                hub.append(("m", qs, m))
    h0, h4 = (len(make_plan(lib, 24, 6, hub, lookahead=la)) for la in (0, 4))
    assert h0 <= 60 and h4 <= 52 and h4 < h0, (h0, h4)


def test_plan_settings_validated(lib):
    """The plan setters accept their documented ranges and refuse the rest
    (and a null plan) with -1."""
    L = lib
    L.quest_gb300_planPassControls.restype = C.c_int
    p = L.quest_gb300_planCreate(20, 6)
    assert L.quest_gb300_planSetLookahead(p, 0) == 0 and L.quest_gb300_planSetLookahead(p, 16) == 0
    assert L.quest_gb300_planSetLookahead(p, -1) == -1 and L.quest_gb300_planSetLookahead(p, 17) == -1
    assert L.quest_gb300_planSetMaxControls(p, 0) == 0 and L.quest_gb300_planSetMaxControls(p, 3) == 0
    assert L.quest_gb300_planSetMaxControls(p, 4) == -1 and L.quest_gb300_planSetMaxControls(p, -1) == -1
    assert L.quest_gb300_planSetBeamWidth(p, 0) == -1
    assert L.quest_gb300_planPassControls(p, 0, None) == -1          # not compiled
    L.quest_gb300_planDestroy(p)
    assert L.quest_gb300_planSetLookahead(None, 4) == -1 and L.quest_gb300_planSetMaxControls(None, 1) == -1


def test_invalid_gates_rejected(lib):
    p = lib.quest_gb300_planCreate(4, 3)
    assert lib.quest_gb300_planAddControlledNot(p, 1, 1) == -1
    assert lib.quest_gb300_planAddControlledNot(p, 1, 4) == -1
    lib.quest_gb300_planDestroy(p)
    assert lib.quest_gb300_planCreate(4, 7) is None


def test_compile_like_reuses_the_passes_with_new_angles(lib):
    """planCompileLike: the same circuit with other angles takes the passes of
    a compiled plan without a search, and its pass products still reproduce
    the new circuit exactly; a circuit of another shape is refused."""
    L = lib
    L.quest_gb300_planCompileLike.argtypes = [C.c_void_p, C.c_void_p]
    n, kmax = 9, 4
    ops_a = W.c2_circuit(n=n, layers=4, seed=21)
    # the same gates on the same qubits, other angles
    ops_b = [op if op[0] != "cu" else (op[0], op[1]) + tuple(np.roll(op[2:], 1)) for op in ops_a]
    ops_b = [op if op[0] != "cp" else (op[0], op[1], op[2], op[3] + 0.7) for op in ops_b]

    def build(ops):
        p = L.quest_gb300_planCreate(n, kmax)
        for op in ops:
            if op[0] == "cu":
                assert L.quest_gb300_planAddCompactUnitary(p, *op[1:]) == 0
            elif op[0] == "cx":
                assert L.quest_gb300_planAddControlledNot(p, op[1], op[2]) == 0
            elif op[0] == "cp":
                assert L.quest_gb300_planAddControlledPhaseShift(p, op[1], op[2], op[3]) == 0
        return p

    pa, pb = build(ops_a), build(ops_b)
    na = L.quest_gb300_planCompile(pa)
    assert na > 0
    assert L.quest_gb300_planCompileLike(pb, pa) == na
    psi = np.zeros(1 << n, dtype=complex)
    psi[0] = 1
    for i in range(na):
        t = (C.c_int * 6)()
        re, im = np.zeros(4096), np.zeros(4096)
        k = L.quest_gb300_planPass(pb, i, t, re.ctypes.data_as(C.POINTER(C.c_double)), im.ctypes.data_as(C.POINTER(C.c_double)))
        D = 1 << k
        psi = apply_matrix(psi, n, list(t[:k]), (re[:D * D] + 1j * im[:D * D]).reshape(D, D))
    want = reference(n, ops_b)
    assert np.max(np.abs(psi - want)) < 1e-12
    # another shape: one gate fewer
    pc = build(ops_b[:-1])
    assert L.quest_gb300_planCompileLike(pc, pa) == -1
    for p in (pa, pb, pc):
        L.quest_gb300_planDestroy(p)
