"""Batched swap tests against the FP64 closed form (1 + <u|v>^2) / 2, against
the same circuit run gate by gate through the QuEST API (FP64), and against
the oracle for small registers."""
import ctypes as C

import numpy as np
import pytest

from quantumlab_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def make_batch(L, pool, offsets, dims, ia, ib):
    P = lambda a, t: a.ctypes.data_as(C.POINTER(t))
    h = L.lib.quest_gb300_swapTestBatchCreate(P(pool, C.c_double), P(offsets, C.c_longlong), P(dims, C.c_int),
                                              len(offsets), P(ia, C.c_int), P(ib, C.c_int), len(ia))
    assert h
    return h


def test_swap_batch_closed_form_all_sizes(gpulib):
    L = gpulib
    rng = np.random.default_rng(7)
    vecs = []
    for d in range(1, 11):
        for _ in range(4):
            v = rng.normal(size=1 << d)
            vecs.append(v / np.linalg.norm(v))
    dims = np.array([int(np.log2(len(v))) for v in vecs], dtype=np.int32)
    offsets = np.cumsum([0] + [len(v) for v in vecs[:-1]]).astype(np.int64)
    pool = np.concatenate(vecs)
    ia, ib = [], []
    for i in range(len(vecs)):
        for j in range(len(vecs)):
            if dims[i] == dims[j]:
                ia.append(i)
                ib.append(j)
    ia, ib = np.array(ia, dtype=np.int32), np.array(ib, dtype=np.int32)
    h = make_batch(L, pool, offsets, dims, ia, ib)
    out = np.zeros(len(ia))
    for _ in range(2):                     # graph replay twice
        assert L.lib.quest_gb300_swapTestBatchRun(h, out.ctypes.data_as(C.POINTER(C.c_double))) == 0
        want = np.array([(1 + np.dot(vecs[a], vecs[b]) ** 2) / 2 for a, b in zip(ia, ib)])
        err = np.max(np.abs(out - want))
        print(f"max |P0 - closed form| = {err:.2e}")
        assert err < 1e-6
    L.lib.quest_gb300_swapTestBatchDestroy(h)


def test_swap_batch_matches_per_gate_circuit(gpulib, oracle):
    L = gpulib
    ds, comps, vecs, cents = W.gaussian_mixture_vectors(count=24, dmin=2, dmax=7, seed=9)
    pool, offsets, dims, ia, ib = W.swap_test_pool(vecs, cents, dmin=2, dmax=7)
    sel = np.arange(0, len(ia), 7)
    ia, ib = ia[sel], ib[sel]
    h = make_batch(L, pool, offsets, dims, ia, ib)
    out = np.zeros(len(ia))
    assert L.lib.quest_gb300_swapTestBatchRun(h, out.ctypes.data_as(C.POINTER(C.c_double))) == 0
    L.lib.quest_gb300_swapTestBatchDestroy(h)
    items = list(vecs) + [m for d in range(2, 8) for m in cents[d]]
    regs = {}
    for k, (a, b) in enumerate(zip(ia, ib)):
        d = int(dims[a])
        u, v = items[a], items[b]
        for lib in (L, oracle) if d <= 5 else (L,):
            key = (id(lib), d)
            if key not in regs:
                regs[key] = lib.create(2 * d + 1)
            p_gate = W.swap_test_plain(lib, regs[key], u, v, d)
            assert abs(p_gate - (1 + np.dot(u, v) ** 2) / 2) < 1e-12
            assert abs(out[k] - p_gate) < 1e-6


def test_swap_batch_tuning_keeps_results(gpulib):
    """swapTestBatchTune tries every CTAs-per-SM / shared-memory threshold
    pairing, keeps the fastest, and the batch still matches the closed form
    (sizes on both sides of every threshold: d = 2 .. 8)."""
    L = gpulib
    rng = np.random.default_rng(11)
    vecs = []
    for d in range(2, 9):
        for _ in range(3):
            v = rng.normal(size=1 << d)
            vecs.append(v / np.linalg.norm(v))
    dims = np.array([int(np.log2(len(v))) for v in vecs], dtype=np.int32)
    offsets = np.cumsum([0] + [len(v) for v in vecs[:-1]]).astype(np.int64)
    pool = np.concatenate(vecs)
    pairs = [(a, b) for a in range(len(vecs)) for b in range(len(vecs)) if dims[a] == dims[b]]
    ia = np.array([a for a, _ in pairs], dtype=np.int32)
    ib = np.array([b for _, b in pairs], dtype=np.int32)
    h = make_batch(L, pool, offsets, dims, ia, ib)
    c, s, best, dflt = C.c_int(0), C.c_int(0), C.c_double(0), C.c_double(0)
    assert L.lib.quest_gb300_swapTestBatchTune(h, C.byref(c), C.byref(s), C.byref(best), C.byref(dflt)) == 0
    assert 2 <= c.value <= 4 and s.value in (512, 2048, 8192) and 0 < best.value <= dflt.value
    out = np.zeros(len(ia))
    assert L.lib.quest_gb300_swapTestBatchRun(h, out.ctypes.data_as(C.POINTER(C.c_double))) == 0
    want = np.array([(1 + np.dot(vecs[a], vecs[b]) ** 2) / 2 for a, b in pairs])
    assert np.max(np.abs(out - want)) < 1e-6
    L.lib.quest_gb300_swapTestBatchDestroy(h)
