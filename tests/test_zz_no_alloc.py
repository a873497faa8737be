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


def test_no_alloc_rejects_oversized_misaligned_and_invalid(gpulib):
    """Sizes beyond the fixed scratch, sizes that are not powers of two and
    arrays that do not start on a 16-byte boundary (an odd offset into a
    register) are rejected on the host, before anything reaches the GPU."""
    L = gpulib
    assert L.capture_errors()
    q = L.create(4)
    L.lib.initDebugState(q)
    amps = L.amps(q)
    L.errors.clear()
    out = C.c_double(-1.0)
    p = C.cast(q.deviceStateVec.real, C.c_void_p), C.cast(q.deviceStateVec.imag, C.c_void_p)
    assert L.lib.quest_gb300_calcTotalProbNoAlloc(p[0], p[1], 1 << 28, C.byref(out), None) != 0
    assert L.lib.quest_gb300_calcTotalProbNoAlloc(p[0], p[1], 12, C.byref(out), None) != 0
    odd = C.c_void_p(p[0].value + 8), C.c_void_p(p[1].value + 8)        # real + 1, imag + 1
    assert L.lib.quest_gb300_calcTotalProbNoAlloc(odd[0], p[1], 8, C.byref(out), None) != 0
    assert L.lib.quest_gb300_calcTotalProbNoAlloc(p[0], odd[1], 8, C.byref(out), None) != 0
    msgs = [m for _, m in L.errors]
    assert len(msgs) == 4 and "2^27" in msgs[0] and "16-byte" in msgs[2] and "16-byte" in msgs[3]
    assert out.value == -1.0
    rc, got = _call(L, q, 16)                   # still usable afterwards
    assert rc == 0 and abs(got - float(np.sum(np.abs(amps) ** 2))) < 1e-12
    even = C.c_void_p(p[0].value + 16), C.c_void_p(p[1].value + 16)      # real + 2: aligned, accepted
    rc = L.lib.quest_gb300_calcTotalProbNoAlloc(even[0], even[1], 8, C.byref(out), None)
    assert rc == 0 and abs(out.value - float(np.sum(np.abs(amps[2:10]) ** 2))) < 1e-12
    L.destroy(q)


def test_no_alloc_allocates_nothing(gpulib):
    """After one warm-up call per size (which may load the kernel's code), the
    device's free memory is the same before and after further calls, up to
    the largest size the entry point takes (27 qubits)."""
    torch = pytest.importorskip("torch")
    L = gpulib
    regs = [L.create(n) for n in (5, 27)]
    for q in regs:
        L.lib.initPlusState(q)
        assert _call(L, q, q.numAmpsTotal)[0] == 0
    free_before = torch.cuda.mem_get_info(0)[0]
    for _ in range(3):
        for q in regs:
            rc, got = _call(L, q, q.numAmpsTotal)
            assert rc == 0 and abs(got - 1.0) < 1e-12
    assert torch.cuda.mem_get_info(0)[0] == free_before
    for q in regs:
        L.destroy(q)
