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
    L.quest_gb300_planCompile.argtypes = [C.c_void_p]
    L.quest_gb300_planPass.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double), C.POINTER(C.c_double)]
    return L


def make_plan(L, n, kmax, ops):
    p = L.quest_gb300_planCreate(n, kmax)
    for op in ops:
        if op[0] == "cu":
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
        passes.append((list(t[:k]), (re[:D * D] + 1j * im[:D * D]).reshape(D, D)))
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
    for op in ops:
        if op[0] == "cu":
            a, b = complex(op[2], op[3]), complex(op[4], op[5])
            psi = apply_matrix(psi, n, [op[1]], np.array([[a, -b.conjugate()], [b, a.conjugate()]]))
        elif op[0] == "cx":
            m = np.eye(4)[[0, 3, 2, 1]]
            psi = apply_matrix(psi, n, [op[1], op[2]], m)
        elif op[0] == "cp":
            psi = apply_matrix(psi, n, [op[1], op[2]], np.diag([1, 1, 1, np.exp(1j * op[3])]))
    return psi


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


def test_plan_pass_count_30q(lib):
    ops = W.c2_circuit(n=30, layers=20, seed=2)
    counts = {k: len(make_plan(lib, 30, k, ops)) for k in (4, 5, 6)}
    # plain per-gate execution would need 1190 passes
    assert counts[4] < 260 and counts[5] < 220 and counts[6] < 180, counts
    assert counts[6] <= counts[5] <= counts[4]


def test_invalid_gates_rejected(lib):
    p = lib.quest_gb300_planCreate(4, 3)
    assert lib.quest_gb300_planAddControlledNot(p, 1, 1) == -1
    assert lib.quest_gb300_planAddControlledNot(p, 1, 4) == -1
    lib.quest_gb300_planDestroy(p)
    assert lib.quest_gb300_planCreate(4, 7) is None
