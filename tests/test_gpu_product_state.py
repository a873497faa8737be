"""quest_gb300_initProductState (GPU): the product of normalised register
vectors, written in one pass, must equal initStateFromAmps of their
Kronecker product; prepared as |0>|v>|u>, the swap-test circuit run on it
through the QuEST API gives P(0) = (1 + |<u|v>|^2) / 2."""
import ctypes as C
import time

import numpy as np
import pytest

from quantumlab_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.fixture(autouse=True)
def no_library_errors(gpulib):
    gpulib.capture_errors()
    gpulib.errors.clear()
    yield
    errors = list(gpulib.errors)
    gpulib.errors.clear()
    assert not errors, errors


def test_product_state_matches_kron(gpulib):
    L = gpulib
    rng = np.random.default_rng(4)
    n, dims = 14, [3, 5, 2]                          # registers on qubits 0-2, 3-7, 8-9; 10-13 |0>
    vecs = [rng.normal(size=1 << d) + 1j * rng.normal(size=1 << d) for d in dims]
    flat = np.concatenate(vecs)
    re, im = np.ascontiguousarray(flat.real), np.ascontiguousarray(flat.imag)
    q = L.create(n)
    regs = (C.c_int * len(dims))(*dims)
    assert L.lib.quest_gb300_initProductState(q, len(dims), regs, dptr(re), dptr(im)) == 0
    want = np.array([1.0 + 0j])
    for v in vecs:
        want = np.kron(v / np.linalg.norm(v), want)  # register r above the previous ones
    want = np.concatenate([want, np.zeros((1 << n) - want.size)])
    got = L.amps(q)
    assert np.max(np.abs(got - want)) < 1e-14
    # real vectors: im may be NULL
    assert L.lib.quest_gb300_initProductState(q, 1, (C.c_int * 1)(3), dptr(np.ascontiguousarray(vecs[0].real)), None) == 0
    r0 = vecs[0].real / np.linalg.norm(vecs[0].real)
    assert np.max(np.abs(L.amps(q)[:8] - r0)) < 1e-15 and np.all(L.amps(q)[8:] == 0)
    L.destroy(q)


def test_product_state_feeds_the_swap_test(gpulib):
    L = gpulib
    rng = np.random.default_rng(8)
    d = 4
    u, v = rng.normal(size=1 << d), rng.normal(size=1 << d)
    q = L.create(2 * d + 1)
    flat = np.ascontiguousarray(np.concatenate([u, v]))
    assert L.lib.quest_gb300_initProductState(q, 2, (C.c_int * 2)(d, d), dptr(flat), None) == 0
    p0 = W.swap_test_plain(L, q, u / np.linalg.norm(u), v / np.linalg.norm(v), d, prepared=True)
    un, vn = u / np.linalg.norm(u), v / np.linalg.norm(v)
    assert abs(p0 - (1 + np.dot(un, vn) ** 2) / 2) < 1e-12
    L.destroy(q)


def test_product_state_rejects_bad_registers(gpulib):
    L = gpulib
    q = L.create(6)
    z = np.zeros(8)
    assert L.lib.quest_gb300_initProductState(q, 1, (C.c_int * 1)(3), dptr(z), None) == -1
    assert L.lib.quest_gb300_initProductState(q, 2, (C.c_int * 2)(4, 3), dptr(np.ones(24)), None) == -1
    assert len(L.errors) == 2
    L.errors.clear()
    L.destroy(q)


def test_product_state_timing_against_kron_upload(gpulib):
    """Wall time to prepare |v>|u> on 24 qubits (two 12-qubit registers):
    the host Kronecker product uploaded with initStateFromAmps against one
    initProductState call; both give the same state (printed; -s)."""
    L = gpulib
    rng = np.random.default_rng(12)
    d, n = 12, 24
    u, v = rng.normal(size=1 << d), rng.normal(size=1 << d)
    u, v = u / np.linalg.norm(u), v / np.linalg.norm(v)
    flat = np.ascontiguousarray(np.concatenate([u, v]))
    regs = (C.c_int * 2)(d, d)
    q = L.create(n)
    times = {}
    for side in ("kron", "product", "kron", "product"):       # second round timed
        L.lib.syncQuESTEnv(L.env)
        t0 = time.perf_counter()
        if side == "kron":
            L.set_amps(q, np.kron(v, u))
        else:
            assert L.lib.quest_gb300_initProductState(q, 2, regs, dptr(flat), None) == 0
        L.lib.syncQuESTEnv(L.env)
        times[side] = (time.perf_counter() - t0) * 1e3
        if side == "kron":
            want = L.amps(q)
        else:
            assert np.max(np.abs(L.amps(q) - want)) < 1e-15
    print(f"\n{n} qubits from two {d}-qubit vectors: kron + initStateFromAmps {times['kron']:.1f} ms, "
          f"initProductState {times['product']:.3f} ms ({times['kron'] / times['product']:.0f}x)")
    L.destroy(q)
