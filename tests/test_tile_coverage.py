"""The pipelined tensor-core kernel's addressing, checked on the host (no
GPU): quest_gb300_checkTileCoverage walks every CTA, tile, warp and lane of a
pass from the launch parameters the kernel receives, with the loaders' and
the epilogue's tile sequences, and reports whether every amplitude is read
and written exactly once.  Covers target layouts of every class (targets
above qubit 5, some below, qubits 0 and 1 among them), control qubits, and
the passes of compiled plans."""
import ctypes as C

import numpy as np
import pytest

import quantumlab_gb300 as qg
from quantumlab_gb300 import workloads as W


@pytest.fixture(scope="module")
def L():
    return qg.load()


def coverage(L, n, targets, controls=()):
    t = (C.c_int * len(targets))(*targets)
    c = (C.c_int * max(1, len(controls)))(*controls)
    return L.lib.quest_gb300_checkTileCoverage(n, t, len(targets), c, len(controls))


@pytest.mark.parametrize("n,targets,controls", [
    (16, [0, 1, 2, 3], []), (16, [5, 6, 7, 8], []), (18, [0, 2, 4, 6, 8], []), (18, [0, 1, 2, 3, 4, 5], []),
    (18, [1, 3, 5, 7, 9, 11], []), (20, [12, 13, 14, 15, 16, 17], []), (20, [0, 1, 9, 17], []),
    (20, [0, 5, 9, 12, 13, 19], []),
    (16, [0, 1, 2, 3], [13]), (18, [5, 6, 7, 8], [15, 16, 17]), (20, [0, 2, 4, 6, 8], [13, 19]),
    (20, [1, 3, 5, 7, 9, 11], [18, 19]), (21, [0, 1, 7, 12, 13, 14], [15, 16, 20]),
    (22, [2, 9, 10, 14, 18, 21], [11, 12, 13]), (19, [12, 13, 14, 15, 16, 17], [7, 18]),
])
def test_every_amplitude_once(L, n, targets, controls):
    assert coverage(L, n, targets, controls) == 0


def test_controls_inside_the_tile_are_refused(L):
    # the 7 lowest non-target qubits belong to the tile: a control there does not fit
    assert coverage(L, 20, [0, 1, 2, 3], [5]) == -1
    assert coverage(L, 20, [8, 9, 10, 11], [3]) == -1
    assert coverage(L, 20, [0, 1, 2, 3], [3]) == -1          # a target
    assert coverage(L, 11, [0, 1, 2, 3], []) == 0
    assert coverage(L, 10, [0, 1, 2, 3], []) == -1           # fewer than k + 7 qubits


def test_passes_of_compiled_plans(L):
    """Every tensor-core pass of the random circuit at 22 and 18 qubits,
    compiled with up to three control qubits per pass."""
    lib = L.lib
    checked = controlled = 0
    for n, ops in ((22, W.c2_circuit(n=22, layers=6, seed=4)), (18, W.c2_circuit(n=18, layers=6, seed=9))):
        p = lib.quest_gb300_planCreate(n, 6)
        assert lib.quest_gb300_planSetMaxControls(p, 3) == 0
        for o in ops:
            if o[0] == "cu":
                lib.quest_gb300_planAddCompactUnitary(p, o[1], o[2], o[3], o[4], o[5])
            elif o[0] == "cx":
                lib.quest_gb300_planAddControlledNot(p, o[1], o[2])
            else:
                lib.quest_gb300_planAddControlledPhaseShift(p, o[1], o[2], o[3])
        npass = lib.quest_gb300_planCompile(p)
        for i in range(npass):
            t = (C.c_int * 6)()
            k = lib.quest_gb300_planPass(p, i, t, None, None)
            cq = (C.c_int * 3)()
            nc = lib.quest_gb300_planPassControls(p, i, cq)
            if k < 4:
                continue
            assert coverage(L, n, list(t[:k]), list(cq[:nc])) == 0, (list(t[:k]), list(cq[:nc]))
            checked += 1
            controlled += nc > 0
        lib.quest_gb300_planDestroy(p)
    assert checked > 10 and controlled > 3


def test_operand_image_layouts(L):
    """Every tensor-core kernel reads its operand part inside the image block
    the library lays out for the parts it built (16-byte aligned, no overlap)."""
    assert L.lib.quest_gb300_checkImageLayouts() == 0


def test_host_half_rounding_matches_ieee(L):
    """The host rounding that builds split-FP16 operand images equals IEEE
    binary16 round-to-nearest-even (numpy's float64 -> float16, one rounding):
    random values over FP16's whole range, its subnormals, exact ties at
    both ends of a binade, and values past the largest finite one."""
    rng = np.random.default_rng(7)
    vals = [rng.normal(size=4000) * np.exp2(rng.integers(-30, 17, size=4000)),
            rng.uniform(-1, 1, size=2000) * 2.0 ** -14,                           # subnormal range
            (np.arange(1, 2049) + 0.5) * 2.0 ** -24,                             # ties on the subnormal grid
            (1024 + np.arange(0, 1024) + 0.5) * 2.0 ** -10,                      # ties in [1, 2)
            np.array([0.0, -0.0, 65504.0, 65519.99, 65520.0, 1e6, -1e6, 2.0 ** -25, 2.0 ** -25 * 1.0000001,
                      6.103515625e-05, 5.960464477539063e-08])]
    v = np.ascontiguousarray(np.concatenate(vals))
    out = np.zeros(v.size, dtype=np.uint16)
    assert L.lib.quest_gb300_roundHalf(v.ctypes.data_as(C.POINTER(C.c_double)),
                                       out.ctypes.data_as(C.POINTER(C.c_ushort)), v.size) == 0
    with np.errstate(over="ignore"):
        want = v.astype(np.float16).view(np.uint16)
    bad = np.nonzero(out != want)[0]
    assert bad.size == 0, [(v[i], hex(out[i]), hex(want[i])) for i in bad[:8]]
    assert L.lib.quest_gb300_roundHalf(None, None, -1) == -1


def test_tensor_core_precision_modes(L):
    """setTensorCorePrecision takes 0 (split-TF32), 1 (split-BF16) and 2
    (split-FP16) and refuses other modes (host state only, no GPU)."""
    lib = L.lib
    before = lib.quest_gb300_getTensorCorePrecision()
    try:
        for mode in (0, 1, 2):
            assert lib.quest_gb300_setTensorCorePrecision(mode) == 0
            assert lib.quest_gb300_getTensorCorePrecision() == mode
        for bad in (-1, 3):
            assert lib.quest_gb300_setTensorCorePrecision(bad) == -1
            assert lib.quest_gb300_getTensorCorePrecision() == 2
    finally:
        lib.quest_gb300_setTensorCorePrecision(before)


def test_split_fp16_images_encode_their_blocks(L):
    """The split-FP16 operand images (two FP16 parts of 2^s G and the factor
    2^-(14 + s) after them) give every entry of matrix blocks from zero to
    1e4 in size back to 2^-21 of the block's largest entry."""
    assert L.lib.quest_gb300_checkHalfImages() == 0
