"""quest_gb300_calcTotalProbNoAlloc: the total probability of caller-owned
device arrays with scratch in a fixed __device__ array instead of
cudaMalloc -- for callers that must not allocate while they run.

Collected last (file name) so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(L, q, n_amps):
    out = C.c_double(-1.0)
    rc = L.lib.quest_gb300_calcTotalProbNoAlloc(C.cast(q.deviceStateVec.real, C.c_void_p),
                                                C.cast(q.deviceStateVec.imag, C.c_void_p),
                                                n_amps, C.byref(out), None)
    return rc, out.value


@pytest.mark.parametrize("n", [1, 5, 17, 24, 27])
def test_no_alloc_matches_calcTotalProb(gpulib, n):
    L = gpulib
    q = L.create(n)
    rng = np.random.default_rng(100 + n)
    if n <= 20:
        psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        L.set_amps(q, psi * 0.731)              # not normalised: a non-trivial sum
    else:
        L.lib.initPlusState(q)
        L.lib.rotateY(q, 3, 0.4)
        L.lib.phaseShift(q, 5, 0.2)
    want = L.lib.calcTotalProb(q)               # the existing entry point
    for _ in range(2):                          # two calls in a row share the scratch
        rc, got = _call(L, q, 1 << n)
        assert rc == 0
        assert abs(got - want) <= 1e-13 * max(1.0, abs(want)), (n, got, want)
    L.destroy(q)


def test_no_alloc_rejects_oversized_and_invalid(gpulib):
    L = gpulib
    assert L.capture_errors()
    q = L.create(4)
    L.errors.clear()
    out = C.c_double(-1.0)
    p = C.cast(q.deviceStateVec.real, C.c_void_p), C.cast(q.deviceStateVec.imag, C.c_void_p)
    assert L.lib.quest_gb300_calcTotalProbNoAlloc(p[0], p[1], 1 << 28, C.byref(out), None) != 0
    assert L.lib.quest_gb300_calcTotalProbNoAlloc(p[0], p[1], 12, C.byref(out), None) != 0
    assert len(L.errors) == 2 and "2^27" in L.errors[0][1]
    assert out.value == -1.0
    rc, got = _call(L, q, 16)                   # still usable afterwards
    assert rc == 0 and abs(got - 1.0) < 1e-14
    L.destroy(q)
